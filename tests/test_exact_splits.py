"""CPU checks of two arithmetic claims the GPU kernels rest on.

1. The tensor-core layer 1 of the proposal network (csrc/proposal.cu) feeds
   each FP32 coordinate as three bf16 terms hi = bf16(x), mid =
   bf16(x - hi), lo = bf16(x - hi - mid); their sum is x exactly, so the
   layer's products are exact and only the FP32 summation order differs
   from the CUDA-core form.  The max-pooled features go to the head as
   hi + lo (two terms), within 2^-16 relative of the FP32 value.
2. The plane angle gates (csrc/models.cu, plane_gates): FP32 Euler angles of
   FromTwoVectors(z, n) decide the gate only outside a 1e-4 rad margin
   around every branch and threshold, else the FP64 angles decide.  A
   restatement of both in numpy must never disagree where the FP32 path
   claims certainty (sloam.cpp:394-408 for the gate; Eigen's
   Quaternion::setFromTwoVectors + eulerAngles(0, 1, 2) restated in
   euler_two_vectors).
"""
import numpy as np

f32 = np.float32


def bf16(x):
    """Round-to-nearest-even to bf16, returned as float32."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def test_three_term_bf16_split_is_exact():
    rng = np.random.default_rng(0)
    x = np.concatenate([
        (rng.standard_normal(200_000) * 10 ** rng.uniform(-6, 2, 200_000)).astype(f32),
        f32([0.0, -0.0, 1.0, -1.0, 3.0e-8, 65504.0, 1.0 + 2 ** -23]),
    ]).astype(f32)
    hi = bf16(x)
    r1 = (x - hi).astype(f32)
    mi = bf16(r1)
    lo = bf16((r1 - mi).astype(f32))
    assert np.array_equal(hi.astype(np.float64) + mi + lo, x.astype(np.float64))


def test_two_term_bf16_split_bound():
    rng = np.random.default_rng(1)
    h = np.abs(rng.standard_normal(200_000) * 10 ** rng.uniform(-4, 2, 200_000)).astype(f32)
    hh = bf16(h)
    hl = bf16((h - hh).astype(f32))
    err = np.abs(hh.astype(np.float64) + hl - h) / np.maximum(h, 1e-30)
    assert err.max() <= 2.0 ** -16


def _euler64(b):
    v1 = b / np.linalg.norm(b)
    c = v1[2]
    if c < -1 + 1e-12:
        return None
    axis = np.array([-v1[1], v1[0], 0.0])
    s = np.sqrt((1 + c) * 2)
    qx, qy, qz = axis / s
    qw = s * 0.5
    tx, ty, tz = 2 * qx, 2 * qy, 2 * qz
    twx, twy, twz = tx * qw, ty * qw, tz * qw
    txx, txy, txz = tx * qx, ty * qx, tz * qx
    tyy, tyz, tzz = ty * qy, tz * qy, tz * qz
    M00, M01, M02 = 1 - (tyy + tzz), txy - twz, txz + twy
    M10, M11, M12 = txy + twz, 1 - (txx + tzz), tyz - twx
    M20, M21, M22 = txz - twy, tyz + twx, 1 - (txx + tyy)
    r0 = np.arctan2(M12, M22)
    c2 = np.hypot(M00, M01)
    if r0 > 0:
        r0 -= np.pi
        r1 = np.arctan2(-M02, -c2)
    else:
        r1 = np.arctan2(-M02, c2)
    s1, c1 = np.sin(r0), np.cos(r0)
    r2 = np.arctan2(s1 * M20 - c1 * M10, c1 * M11 - s1 * M21)
    return [-r0, -r1, -r2]


def _euler32(b, eps=f32(1e-4)):
    bx, by, bz = (f32(v) for v in b)
    nb = np.sqrt(bx * bx + by * by + bz * bz)
    vx, vy, vz = bx / nb, by / nb, bz / nb
    if not (vz > f32(-1) + f32(1e-5)):
        return None
    s = np.sqrt((f32(1) + vz) * f32(2))
    invs = f32(1) / s
    qx, qy, qz, qw = -vy * invs, vx * invs, f32(0), s * f32(0.5)
    tx, ty, tz = 2 * qx, 2 * qy, 2 * qz
    twx, twy, twz = tx * qw, ty * qw, tz * qw
    txx, txy, txz = tx * qx, ty * qx, tz * qx
    tyy, tyz, tzz = ty * qy, tz * qy, tz * qz
    M00, M01, M02 = f32(1) - (tyy + tzz), txy - twz, txz + twy
    M10, M11 = txy + twz, f32(1) - (txx + tzz)
    M20, M21, M22, M12 = txz - twy, tyz + twx, f32(1) - (txx + tyy), tyz - twx
    PIf = f32(3.14159265)
    r0 = np.arctan2(M12, M22)
    if abs(r0) < eps or abs(PIf - abs(r0)) < eps:
        return None
    c2 = np.hypot(M00, M01)
    if r0 > 0:
        r0 = r0 - PIf
        r1 = np.arctan2(-M02, -c2)
    else:
        r1 = np.arctan2(-M02, c2)
    s1, c1 = np.sin(r0), np.cos(r0)
    r2 = np.arctan2(s1 * M20 - c1 * M10, c1 * M11 - s1 * M21)
    ang = [-r0, -r1, -r2]
    for a in ang:
        if abs(a - f32(0.1)) < eps or abs(PIf - abs(a) - f32(0.1)) < eps:
            return None
    return ang


def _gate(ang, pi):
    return all(a < 0.1 for a in ang) or all(pi - abs(a) < 0.1 for a in ang)


def test_plane_gate_fp32_prefilter_agrees_with_fp64():
    rng = np.random.default_rng(0)
    fast = deferred = 0
    for t in range(20_000):
        if t % 2:  # near-vertical normals, both signs: the gate's border region
            b = np.r_[rng.normal(0, 0.1, 2), 1.0] * rng.choice([1.0, -1.0])
        else:
            b = rng.normal(0, 1, 3)
        a64 = _euler64(b)
        if a64 is None:
            continue
        a32 = _euler32(b)
        if a32 is None:
            deferred += 1
            continue
        fast += 1
        assert _gate(a32, f32(3.14159265)) == _gate(a64, np.pi), (b, a32, a64)
    assert fast > 0.95 * (fast + deferred)
