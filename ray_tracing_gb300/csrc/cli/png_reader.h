// Minimal PNG reader for 8-bit, non-interlaced grey, RGB and RGBA images (the
// ReSTIR acceptance goldens): chunk walk, zlib inflate (RFC 1950/1951: stored,
// fixed and dynamic Huffman blocks) and the five scanline filters, returning
// RGB bytes. No external library.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

namespace rtgb::png {

namespace detail {

struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    uint32_t bits(int k) {
        while (bitcnt < k) {
            if (pos >= n) throw std::runtime_error("png: truncated deflate stream");
            bitbuf |= static_cast<uint32_t>(p[pos++]) << bitcnt;
            bitcnt += 8;
        }
        const uint32_t v = bitbuf & ((k == 32) ? 0xffffffffu : ((1u << k) - 1u));
        bitbuf >>= k;
        bitcnt -= k;
        return v;
    }
    void align() {
        bitbuf = 0;
        bitcnt = 0;
    }
};

// Canonical Huffman decoding table: counts per length and symbols by code order.
struct Huffman {
    std::array<uint16_t, 16> count{};
    std::vector<uint16_t> symbol;
    void build(const uint8_t* lengths, int n) {
        count.fill(0);
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        std::array<uint16_t, 16> offs{};
        for (int len = 1; len < 16; ++len) offs[len] = static_cast<uint16_t>(offs[len - 1] + count[len - 1]);
        symbol.assign(static_cast<size_t>(n), 0);
        for (int i = 0; i < n; ++i) {
            if (lengths[i] != 0) symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
        }
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= static_cast<int>(br.bits(1));
            const int c = count[len];
            if (code - c < first) return symbol[static_cast<size_t>(index + (code - first))];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw std::runtime_error("png: bad Huffman code");
    }
};

inline void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    static const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83,
        99, 115, 131, 163, 195, 227, 258};
    static const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
        1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11,
        12, 12, 13, 13};
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 256) {
            out.push_back(static_cast<uint8_t>(sym));
        } else if (sym == 256) {
            return;
        } else {
            const int li = sym - 257;
            if (li >= 29) throw std::runtime_error("png: bad length symbol");
            const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
            const int di = dist.decode(br);
            if (di >= 30) throw std::runtime_error("png: bad distance symbol");
            const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
            if (d > out.size()) throw std::runtime_error("png: distance past the start");
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

// zlib stream (2-byte header, deflate blocks, Adler-32 not checked) -> bytes
inline std::vector<uint8_t> zlib_inflate(const std::vector<uint8_t>& z) {
    if (z.size() < 2 || (z[0] & 0x0f) != 8 || ((z[0] << 8) | z[1]) % 31 != 0) throw std::runtime_error("png: bad zlib header");
    BitReader br{z.data() + 2, z.size() - 2};
    std::vector<uint8_t> out;
    bool last = false;
    while (!last) {
        last = br.bits(1) != 0;
        const uint32_t type = br.bits(2);
        if (type == 0) {
            br.align();
            if (br.pos + 4 > br.n) throw std::runtime_error("png: truncated stored block");
            const size_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            br.pos += 4;
            if (br.pos + len > br.n) throw std::runtime_error("png: truncated stored block");
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            inflate_block(br, lit, dist, out);
        } else if (type == 2) {
            const int hlit = static_cast<int>(br.bits(5)) + 257;
            const int hdist = static_cast<int>(br.bits(5)) + 1;
            const int hclen = static_cast<int>(br.bits(4)) + 4;
            static const uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; ++i) cl[kOrder[i]] = static_cast<uint8_t>(br.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            std::vector<uint8_t> lens(static_cast<size_t>(hlit + hdist), 0);
            for (int i = 0; i < hlit + hdist;) {
                const int sym = clh.decode(br);
                if (sym < 16) {
                    lens[static_cast<size_t>(i++)] = static_cast<uint8_t>(sym);
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (sym == 16) {
                        if (i == 0) throw std::runtime_error("png: repeat with no previous length");
                        val = lens[static_cast<size_t>(i - 1)];
                        rep = 3 + static_cast<int>(br.bits(2));
                    } else if (sym == 17) {
                        rep = 3 + static_cast<int>(br.bits(3));
                    } else {
                        rep = 11 + static_cast<int>(br.bits(7));
                    }
                    if (i + rep > hlit + hdist) throw std::runtime_error("png: code lengths overflow");
                    while (rep-- > 0) lens[static_cast<size_t>(i++)] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens.data(), hlit);
            dist.build(lens.data() + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            throw std::runtime_error("png: reserved block type");
        }
    }
    return out;
}

inline uint32_t be32(const uint8_t* p) {
    return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) | (static_cast<uint32_t>(p[2]) << 8) | p[3];
}

}  // namespace detail

struct Image {
    int width = 0, height = 0;
    std::vector<uint8_t> rgb;  // width * height * 3, rows top to bottom
};

inline Image read_rgb(const std::filesystem::path& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) throw std::runtime_error("failed to open " + path.string());
    const std::vector<uint8_t> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static const uint8_t kSig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    if (d.size() < 8 || !std::equal(kSig, kSig + 8, d.begin())) throw std::runtime_error(path.string() + ": not a PNG");
    Image img;
    int channels = 0;
    std::vector<uint8_t> z;
    for (size_t pos = 8; pos + 12 <= d.size();) {
        const uint32_t len = detail::be32(&d[pos]);
        const std::string type(reinterpret_cast<const char*>(&d[pos + 4]), 4);
        if (pos + 12 + len > d.size()) throw std::runtime_error(path.string() + ": truncated chunk");
        const uint8_t* body = &d[pos + 8];
        if (type == "IHDR") {
            img.width = static_cast<int>(detail::be32(body));
            img.height = static_cast<int>(detail::be32(body + 4));
            const int depth = body[8], color = body[9], interlace = body[12];
            channels = color == 0 ? 1 : (color == 2 ? 3 : (color == 6 ? 4 : 0));
            if (depth != 8 || channels == 0 || interlace != 0) {
                throw std::runtime_error(path.string() + ": only 8-bit non-interlaced grey/RGB/RGBA PNGs are read");
            }
        } else if (type == "IDAT") {
            z.insert(z.end(), body, body + len);
        } else if (type == "IEND") {
            break;
        }
        pos += 12 + len;
    }
    if (img.width <= 0 || img.height <= 0) throw std::runtime_error(path.string() + ": no IHDR");
    const std::vector<uint8_t> raw = detail::zlib_inflate(z);
    const size_t stride = static_cast<size_t>(img.width) * channels;
    if (raw.size() < (stride + 1) * img.height) throw std::runtime_error(path.string() + ": short image data");
    std::vector<uint8_t> pix(stride * img.height);
    for (int y = 0; y < img.height; ++y) {
        const uint8_t filter = raw[(stride + 1) * y];
        const uint8_t* src = &raw[(stride + 1) * y + 1];
        uint8_t* row = &pix[stride * y];
        const uint8_t* up = y > 0 ? &pix[stride * (y - 1)] : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= static_cast<size_t>(channels) ? row[i - channels] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= static_cast<size_t>(channels)) ? up[i - channels] : 0;
            int pred = 0;
            switch (filter) {
                case 0: pred = 0; break;
                case 1: pred = a; break;
                case 2: pred = b; break;
                case 3: pred = (a + b) / 2; break;
                case 4: {
                    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
                    pred = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: throw std::runtime_error(path.string() + ": bad filter type");
            }
            row[i] = static_cast<uint8_t>((src[i] + pred) & 0xff);
        }
    }
    img.rgb.resize(static_cast<size_t>(img.width) * img.height * 3);
    for (size_t p = 0; p < static_cast<size_t>(img.width) * img.height; ++p) {
        for (int k = 0; k < 3; ++k) img.rgb[p * 3 + k] = pix[p * channels + (channels == 1 ? 0 : k)];
    }
    return img;
}

}  // namespace rtgb::png
