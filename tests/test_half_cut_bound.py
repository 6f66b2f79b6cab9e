"""The finder's half-precision exact cut never drops a pair that the FP32
pair-tile kernel counts.

The cut (tiles.cu: exact_cut_half) compares, for offsets from the block box
centre rounded to half precision, dx = h(xj) - h(xi) per component and
r2 = fma(dx, dx, fma(dy, dy, dz * dz)) in half arithmetic against
h((rc + 0.005)^2).  It is used for rows whose block box has half extents
<= 0.75 nm and cutoffs <= 1.5 nm, where the offsets of i atoms are <= 0.75 nm and
those of staged j atoms <= 0.75 + rc per component.  Half arithmetic is emulated
here with numpy float16 (each operation computed exactly in float64, then rounded
once to nearest, as the fused half instructions do)."""
import numpy as np
import pytest

MARGIN = 0.005
MAX_H = 0.75


def h(x):
    return np.asarray(x, dtype=np.float64).astype(np.float16).astype(np.float64)


def half_r2(rj, ri):
    d = h(h(rj) - h(ri))
    t = h(d[:, 2] * d[:, 2])
    t = h(d[:, 1] * d[:, 1] + t)
    return h(d[:, 0] * d[:, 0] + t)


def fp32_r2(rj, ri):
    d = (rj.astype(np.float32) - ri.astype(np.float32)).astype(np.float32)
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(np.float32)


@pytest.mark.parametrize("rc", [0.8, 0.9, 1.0, 1.2, 1.5])
def test_no_pair_inside_the_cutoff_is_cut(rc):
    rng = np.random.default_rng(int(rc * 100))
    n = 400_000
    # i offsets anywhere in the largest box, j at a distance just below rc
    ri = rng.uniform(-MAX_H, MAX_H, size=(n, 3))
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    r = rc - rng.uniform(0.0, 2e-3, size=n) * rng.choice([1.0, 0.1, 0.01], size=n)
    rj = ri + u * r[:, None]
    # the staged j offsets are within rc of the box: clip to the largest possible
    ok = np.all(np.abs(rj) <= MAX_H + rc, axis=1)
    ri, rj = ri[ok], rj[ok]
    inside = fp32_r2(rj, ri) < np.float32(rc) * np.float32(rc)
    rcm = np.float32(rc) + np.float32(MARGIN)
    thr = h(np.float32(rcm * rcm))
    kept = half_r2(rj, ri) < thr
    assert inside.sum() > 1000
    assert np.all(kept[inside]), int((~kept[inside]).sum())


def test_worst_case_magnitudes():
    # offsets at the extremes of the ranges, along the axes and diagonals
    rc = 1.5
    pts = []
    for s in (-1.0, 1.0):
        for ax in range(3):
            ri = np.zeros(3)
            ri[ax] = -s * MAX_H
            for eps in (1e-7, 1e-5, 1e-4, 1e-3):
                rj = ri.copy()
                rj[ax] += s * (rc - eps)
                pts.append((rj, ri))
        d = np.ones(3) / np.sqrt(3.0)
        ri = -s * MAX_H * np.ones(3)
        for eps in (1e-7, 1e-5, 1e-4, 1e-3):
            pts.append((ri + s * d * (rc - eps), ri))
    rj = np.array([p[0] for p in pts])
    ri = np.array([p[1] for p in pts])
    inside = fp32_r2(rj, ri) < np.float32(rc) * np.float32(rc)
    rcm = np.float32(rc) + np.float32(MARGIN)
    kept = half_r2(rj, ri) < h(np.float32(rcm * rcm))
    assert np.all(kept[inside])
