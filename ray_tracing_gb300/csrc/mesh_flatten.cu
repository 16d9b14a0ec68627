// Instanced meshes flattened into the scene's packed triangles (add_v2_mesh,
// realtime_scene_adapter.cpp:289-346, per instance) and the coordinate scale
// of the LBVH padding, on the device.
//
// One thread per output triangle: the instance is found by bisection over
// the instances' first output triangles, the prototype's corner table gives
// the three points, and the arithmetic is the host lowering's, operation for
// operation in double precision (no contraction under --fmad=false), so the
// triangles are the host's bit for bit.
#include "mesh_flatten.cuh"

namespace rtgb {
namespace {

constexpr int kFlattenThreads = 256;

// the last instance whose first output triangle is at or before t (instances
// of empty prototypes share their successor's offset and are skipped)
__device__ __forceinline__ int find_instance(const MeshSetDev& m, long long t) {
    int lo = 0, hi = m.instance_count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (m.instances[mid].out_offset <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void transform_point(const double* w, const double* p, float* out) {
    for (int r = 0; r < 3; ++r) {
        const double l = w[4 * r] * p[0] + w[4 * r + 1] * p[1] + w[4 * r + 2] * p[2];
        out[r] = static_cast<float>(l + w[4 * r + 3]);
    }
}

// inverse-transpose of the linear part applied to n, renormalised; false when
// the length is not finite or at most 1e-12
__device__ __forceinline__ bool transform_normal(const double* a, const double* n, float* out) {
    const double t0 = a[0] * n[0] + a[3] * n[1] + a[6] * n[2];
    const double t1 = a[1] * n[0] + a[4] * n[1] + a[7] * n[2];
    const double t2 = a[2] * n[0] + a[5] * n[1] + a[8] * n[2];
    const double len = sqrt(t0 * t0 + t1 * t1 + t2 * t2);
    if (!isfinite(len) || len <= 1e-12) return false;
    out[0] = static_cast<float>(t0 / len);
    out[1] = static_cast<float>(t1 / len);
    out[2] = static_cast<float>(t2 / len);
    return true;
}

__global__ void __launch_bounds__(kFlattenThreads) k_flatten_meshes(MeshSetDev m, rtgb_triangle* __restrict__ out,
    int* bad_normal) {
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long t = m.first_out + blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; t < m.end_out;
         t += stride) {
        const MeshInstDev& in = m.instances[find_instance(m, t)];
        const MeshProtoDev p = m.prototypes[in.prototype];
        const long long j = p.tri_offset + (t - in.out_offset);
        // corner k of the output triangle is corner slot[k] of the prototype's
        const int slot[3] = {0, in.flip ? 2 : 1, in.flip ? 1 : 2};
        rtgb_triangle tri{};
        const int mat = m.materials[j];
        tri.material_index = mat == RTGB_INSTANCE_MATERIAL ? in.material : mat;
        float* pts[3] = {tri.p0, tri.p1, tri.p2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const long long pt = p.point_offset + m.corners[3 * j + slot[k]];
            transform_point(in.world, m.points + 3 * pt, pts[k]);
        }
        if (p.has_normals) {
            float* nrm[3] = {tri.n0, tri.n1, tri.n2};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (!transform_normal(in.normal_matrix, m.normals + 9 * j + 3 * slot[k], nrm[k])) atomicExch(bad_normal, 1);
            }
            tri.has_vertex_normals = 1;
        }
        if (p.has_texcoords) {
            float* uv[3] = {tri.uv0, tri.uv1, tri.uv2};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                uv[k][0] = static_cast<float>(m.texcoords[6 * j + 2 * slot[k]]);
                uv[k][1] = static_cast<float>(m.texcoords[6 * j + 2 * slot[k] + 1]);
            }
            tri.has_texcoords = 1;
        }
        out[t] = tri;
    }
}

__device__ __forceinline__ float nan_to_zero(float v) { return v == v ? v : 0.0f; }

__global__ void k_scene_scale(DeviceScene d, unsigned* scale_bits) {
    const long long n = static_cast<long long>(d.sphere_count) + d.quad_count + d.triangle_count;
    float m = 0.0f;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (i < d.sphere_count) {
            const rtgb_sphere& s = d.spheres[i];
            for (int k = 0; k < 3; ++k) m = fmaxf(m, nan_to_zero(fabsf(s.center[k]) + fabsf(s.radius)));
        } else if (i < d.sphere_count + d.quad_count) {
            const rtgb_quad& q = d.quads[i - d.sphere_count];
            for (int k = 0; k < 3; ++k) m = fmaxf(m, nan_to_zero(fabsf(q.origin[k]) + fabsf(q.edge_u[k]) + fabsf(q.edge_v[k])));
        } else {
            const rtgb_triangle& t = d.triangles[i - d.sphere_count - d.quad_count];
            for (int k = 0; k < 3; ++k) {
                m = fmaxf(m, nan_to_zero(fabsf(t.p0[k])));
                m = fmaxf(m, nan_to_zero(fabsf(t.p1[k])));
                m = fmaxf(m, nan_to_zero(fabsf(t.p2[k])));
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    // non-negative floats order as their bit patterns
    if ((threadIdx.x & 31) == 0) atomicMax(scale_bits, __float_as_uint(m));
}

}  // namespace

cudaError_t launch_flatten_meshes(const MeshSetDev& set, rtgb_triangle* out, int* bad_normal, int sm_count,
    cudaStream_t stream) {
    const long long n = set.end_out - set.first_out;
    if (n <= 0 || set.instance_count <= 0) return cudaSuccess;
    const long long blocks = std::min<long long>((n + kFlattenThreads - 1) / kFlattenThreads, 8ll * sm_count);
    k_flatten_meshes<<<static_cast<int>(blocks), kFlattenThreads, 0, stream>>>(set, out, bad_normal);
    return cudaGetLastError();
}

cudaError_t launch_scene_scale(const DeviceScene& d, unsigned* scale_bits, int sm_count, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(scale_bits, 0, sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
    const long long n = static_cast<long long>(d.sphere_count) + d.quad_count + d.triangle_count;
    if (n <= 0) return cudaSuccess;
    const long long blocks = std::min<long long>((n + 255) / 256, 8ll * sm_count);
    k_scene_scale<<<static_cast<int>(blocks), 256, 0, stream>>>(d, scale_bits);
    return cudaGetLastError();
}

}  // namespace rtgb
