"""|k'_perp|^2 / |k|^2 for disks and Gaussians in FP32, as the kernels form it,
against FP64 on directions close to the normal.

The reference forms |k'|^2 - (k'.n)^2.  In FP32 that difference carries
~1e-7 of rounding at any angle to the normal, and the disk's Bessel argument
x = k rho sqrt(perp) is then off by (k rho)^2 1e-7 / (2 x).  The kernels form
qd (1 - |n|^2) + |n|^2 |v x n/|n||^2 (v = A^T d, qd = |v|^2) with the unit
normal and 1 - |n|^2 precomputed in FP64; its rounding shrinks with the angle.
The test emulates both forms with numpy float32 arithmetic."""
import numpy as np

f32 = np.float32


def perp_difference(v, n):
    v = v.astype(f32)
    n = n.astype(f32)
    qd = (v * v).sum(axis=-1, dtype=f32)
    sn = (v * n).sum(axis=-1, dtype=f32)
    return np.maximum(qd - sn * sn, f32(0))


def perp_cross(v, n64):
    nn = (n64 * n64).sum(axis=-1)
    nhat = (n64 / np.sqrt(nn)[..., None]).astype(f32)
    en = (1.0 - nn).astype(f32)
    v = v.astype(f32)
    qd = (v * v).sum(axis=-1, dtype=f32)
    c = np.cross(v, nhat).astype(f32)
    return qd * en + (f32(1) - en) * (c * c).sum(axis=-1, dtype=f32)


def exact(v, n64):
    v = v.astype(np.float64)
    return (v * v).sum(axis=-1) - ((v * n64).sum(axis=-1)) ** 2


def near_normal_cases(rng, n_cases, unit=True):
    n = rng.normal(size=(n_cases, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    if not unit:
        n *= rng.uniform(0.5, 1.5, size=(n_cases, 1))
    t = rng.normal(size=(n_cases, 3))
    t -= (t * n).sum(1, keepdims=True) * n / (n * n).sum(1, keepdims=True)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    ang = 10.0 ** rng.uniform(-6, -1, size=(n_cases, 1))  # 1e-6 .. 0.1 rad from the normal
    nh = n / np.linalg.norm(n, axis=1, keepdims=True)
    d = np.cos(ang) * nh + np.sin(ang) * t
    return d, n, ang[:, 0]


def test_cross_form_error_shrinks_with_the_angle():
    rng = np.random.default_rng(0)
    d, n, ang = near_normal_cases(rng, 20000)
    ref = exact(d, n)
    kr = 550.0  # k rho at the largest radius of the 64-radius grid for a 0.3-radius disk
    x_ref = kr * np.sqrt(ref)
    x_diff = kr * np.sqrt(perp_difference(d, n).astype(np.float64))
    x_cross = kr * np.sqrt(perp_cross(d, n).astype(np.float64))
    err_diff = np.abs(x_diff - x_ref)
    err_cross = np.abs(x_cross - x_ref)
    # the cross form: Bessel argument within ~kr * 3e-7 rad at every angle
    assert err_cross.max() < kr * 3e-7, err_cross.max()
    # the difference form: errors of 1e-3 rad and more close to the normal
    assert err_diff.max() > 1e-3, err_diff.max()
    # the cross form's perp error scales with sin(angle) = sqrt(perp): the FP32
    # unit normal is turned by ~6e-8 rad, no more
    pc = perp_cross(d, n).astype(np.float64)
    assert np.all(np.abs(pc - ref) <= 3e-7 * np.sqrt(ref) + 1e-14), np.max(np.abs(pc - ref) / np.sqrt(ref))


def test_cross_form_matches_the_reference_for_non_unit_normals():
    """1 - |n|^2 carries the reference's difference for any normal length."""
    rng = np.random.default_rng(1)
    d, n, _ = near_normal_cases(rng, 5000, unit=False)
    v = d * rng.uniform(0.5, 2.0, size=(len(d), 1))  # A^T d of an affine object
    ref = exact(v, n)
    got = perp_cross(v, n).astype(np.float64)
    scale = (v * v).sum(1)
    assert np.max(np.abs(got - ref) / scale) < 1e-6
