"""The form-factor kernel's table phasor e^{i x} (dfmath.cuh: cis_tab_df,
cis_tab_f), emulated in FP32 on the host and held against e^{i x} in FP64.

x = 2 pi kt sm / 256 with kt = k 256 / (2 pi) and sm a direction dot product,
both double-float; y = kt sm is split into n = round(y) (256 table entries
rounded once from FP64) and |f| <= 1/2, with two-term Taylor polynomials for
cos and sin of 2 pi f / 256.  The bound checked, 1.5e-7 per component over
|x| up to 1e5 rad, is the FP32 rounding level of a unit phasor (measured:
8.7e-8 worst, 2.9e-8 rms).  FMAs are
emulated exactly: a product of two FP32 values is exact in FP64 and the sum
with a third rounds once to FP64 before the final rounding to FP32, which
differs from a fused FMA only in ties far below this bound.
"""
import numpy as np

f32 = np.float32
TURN = f32(2 * np.pi / 256)
C2 = f32((2 * np.pi / 256) ** 2 / 2)
C3 = f32((2 * np.pi / 256) ** 3 / 6)
SHIFT = f32(12582912.0)
TAB = np.stack([np.cos(2 * np.pi * np.arange(256) / 256), np.sin(2 * np.pi * np.arange(256) / 256)], 1).astype(f32)


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split(v):
    hi = f32(v)
    return hi, f32(v - np.float64(hi))


def cis_tab_frac(idx, f):
    f2 = f32(f * f)
    cm = f32(f2 * -C2)
    sn = f32(f * fma(f2, -C3, TURN))
    tx, ty = TAB[idx]
    return fma(tx, cm, fma(-ty, sn, tx)), fma(ty, cm, fma(tx, sn, ty))


def cis_tab_df(kt, sm):
    t = fma(kt[0], sm[0], SHIFT)  # the exact product rounded to an integer by the shift
    n = f32(t - SHIFT)
    fr = fma(kt[0], sm[0], -n)
    fr = fma(kt[0], sm[1], fr)
    fr = fma(kt[1], sm[0], fr)
    idx = int(np.array(t, dtype=f32).view(np.int32)) & 255
    return cis_tab_frac(idx, fr)


def test_table_phasor_error_over_the_phase_range():
    rng = np.random.default_rng(0)
    worst = 0.0
    for _ in range(4000):
        k = 10 ** rng.uniform(-2, 3.9)                    # radii of the workload grids (k up to ~7.3e3)
        s = rng.uniform(-1, 1) * 10 ** rng.uniform(-3, 1.1)  # direction dots up to ~13
        if abs(k * s) > 1.0e5:
            continue
        kt = split(k * 256 / (2 * np.pi))
        sm = split(s)
        x = 2 * np.pi / 256 * (np.float64(kt[0]) + np.float64(kt[1])) * (np.float64(sm[0]) + np.float64(sm[1]))
        re, im = cis_tab_df(kt, sm)
        worst = max(worst, abs(np.float64(re) - np.cos(x)), abs(np.float64(im) - np.sin(x)))
    assert worst <= 1.5e-7, worst


def test_table_index_wraps_for_negative_phases():
    for y in (-1.0, -255.6, -256.0, -1e6 + 0.3, 3.49, 2 ** 21 + 7.0):
        kt, sm = split(y), (f32(1.0), f32(0.0))
        re, im = cis_tab_df(kt, sm)
        x = 2 * np.pi * y / 256
        assert abs(re - np.cos(x)) <= 1.5e-7 and abs(im - np.sin(x)) <= 1.5e-7, y
