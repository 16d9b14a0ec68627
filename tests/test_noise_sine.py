"""The noise texture's sine (ray_tracing_gb300/csrc/noise_sin.h), CPU.

The reference's hash noise multiplies sin(dot(p, k)) by 43758.5453 and keeps
the fraction, so a one-ulp change of the sine moves the hash by ~3e-3. The
kernels and the oracle therefore share one single-precision sine built from
correctly rounded operations only. Here it is checked against the exact sine
(double precision, rounded to float): within 1 ulp for |x| < 2^17, the range
the room scene's noise reaches, and within 2e-7 absolutely up to 2^22."""
import numpy as np


def _ulps(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, 0x80000000 - ia, ia)
    ib = np.where(ib < 0, 0x80000000 - ib, ib)
    return np.abs(ia - ib)


def test_noise_sine_accuracy():
    from oracle.binding import load
    lib = load()
    rng = np.random.default_rng(3)
    for hi, max_ulp, max_abs in ((17, 1, 1e-7), (22, 3, 2e-7)):
        e = rng.uniform(-12.0, hi, 60000)
        x = (np.sign(rng.uniform(-1, 1, e.size)) * np.exp2(e)).astype(np.float32)
        got = np.array([lib.orc_noise_sinf(float(v)) for v in x], dtype=np.float32)
        exact = np.sin(x.astype(np.float64))
        assert np.max(np.abs(got - exact)) <= max_abs
        assert _ulps(got, exact.astype(np.float32)).max() <= max_ulp


def test_noise_sine_quadrants_and_symmetry():
    from oracle.binding import load
    lib = load()
    for x in (0.0, 0.5, 1.0, 2.0, 3.0, 4.0, 5.5, 100.25, 12345.678):
        assert lib.orc_noise_sinf(-x) == -lib.orc_noise_sinf(x)
        assert abs(lib.orc_noise_sinf(x) - np.sin(np.float64(np.float32(x)))) < 1e-7
