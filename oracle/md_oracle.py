"""FP64 CPU restatement of the Langevin MD step the GPU driver takes.

TEST INFRASTRUCTURE ONLY.  Imported by tests/ (and nothing in the product).

It follows, term by term, what the reference's test and examples integrate
(python/tests/test_abfe.py:55-103, example/abfe/abfe.py:94-101): OpenMM's
LangevinIntegrator in its leapfrog form

    a = exp(-gamma dt)
    v <- a v + (1 - a)/gamma f/m + sqrt(kT (1 - a^2)/m) N(0, 1)     ((1 - a)/gamma -> dt at gamma = 0)
    x' = x + dt v;  SHAKE x' against x;  v <- (x' - x)/dt;  x <- x'

over group-0 terms (harmonic bonds and angles, the flat-bottom centroid
restraint of ATMMetaForceUtils.addVsiteRestraintForceCMCM,
python/ATMMetaForceUtils.py:79-138, and the flat-bottom position restraints of
addPosRestraints, :707-752) plus the ATM force.  The normals come from
Philox4x32-10 (Salmon et al., SC'11) with counter (atom index within the
replica, step low, step high, replica << 1 | stream) and key (seed low, seed
high), through Box-Muller in FP32, as on the GPU (CUDA's logf and sincospif
against numpy's float32 log and rounded FP64 cos/sin: equal to 1-2 ulp).
"""
from __future__ import annotations

import math

import numpy as np

KB = 0.00831446261815324  # kJ/mol/K
M32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: (..., 4) uint32-valued array; key: (..., 2).  Returns (..., 4) uint64 holding 32-bit words."""
    c = [np.asarray(ctr[..., k], dtype=np.uint64) for k in range(4)]
    k0 = np.asarray(key[..., 0], dtype=np.uint64) & M32
    k1 = np.asarray(key[..., 1], dtype=np.uint64) & M32
    M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
    W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & M32
        hi1, lo1 = p1 >> np.uint64(32), p1 & M32
        c = [(hi1 ^ c[1] ^ k0) & M32, lo1, (hi0 ^ c[3] ^ k1) & M32, lo0]
        k0 = (k0 + W0) & M32
        k1 = (k1 + W1) & M32
    return np.stack(c, axis=-1)


def normals3(n, step, stream, seed, replica=0):
    """(n, 3) standard normals for atoms 0..n-1 of one replica at one step:
    Box-Muller in FP32 on 24-bit uniforms ((r >> 8) + 0.5) / 2^24, as the GPU draws them."""
    i = np.arange(n, dtype=np.uint64)
    ctr = np.stack([i, np.full(n, step & 0xFFFFFFFF, np.uint64), np.full(n, (step >> 32) & 0xFFFFFFFF, np.uint64),
                    np.full(n, (replica << 1) | stream, np.uint64)], axis=-1)
    key = np.array([seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF], dtype=np.uint64)
    r = philox4x32_10(ctr, np.broadcast_to(key, (n, 2)))
    u = ((r >> np.uint64(8)).astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / 16777216.0)
    a = np.sqrt(np.float32(-2.0) * np.log(u[:, 0]))
    b = np.sqrt(np.float32(-2.0) * np.log(u[:, 2]))
    c1 = np.cos(np.pi * (2.0 * u[:, 1].astype(np.float64))).astype(np.float32)
    s1 = np.sin(np.pi * (2.0 * u[:, 1].astype(np.float64))).astype(np.float32)
    c3 = np.cos(np.pi * (2.0 * u[:, 3].astype(np.float64))).astype(np.float32)
    return np.stack([a * c1, a * s1, b * c3], axis=1).astype(np.float64)


RNG_THERMOSTAT, RNG_VELOCITIES = 0, 1


def group0(pos, terms, box):
    """Energy and forces of the bonds, angles, position and centroid restraints."""
    F = np.zeros_like(pos)
    E = 0.0
    for i, j, r0, k in terms.bonds:
        d = pos[j] - pos[i]
        r = math.sqrt(float(d @ d))
        E += 0.5 * k * (r - r0) ** 2
        f = k * (r - r0) / r * d
        F[i] += f
        F[j] -= f
    for i, j, l, t0, k in terms.angles:
        r1, r2 = pos[i] - pos[j], pos[l] - pos[j]
        cp = np.cross(r1, r2)
        ncp = math.sqrt(float(cp @ cp))
        th = math.atan2(ncp, float(r1 @ r2))
        E += 0.5 * k * (th - t0) ** 2
        if ncp > 0:
            dE = k * (th - t0)
            fi = -dE * np.cross(r1, cp) / (float(r1 @ r1) * ncp)
            fl = dE * np.cross(r2, cp) / (float(r2 @ r2) * ncp)
            F[i] += fi
            F[l] += fl
            F[j] -= fi + fl
    for p in terms.posres_particles:
        d = pos[p] - terms.posres_ref[p]
        if terms.posres_periodic:
            d = d - box * np.rint(d / box)
        r = math.sqrt(float(d @ d))
        if r > terms.posres_tol:
            E += 0.5 * terms.posres_fc * (r - terms.posres_tol) ** 2
            F[p] -= terms.posres_fc * (r - terms.posres_tol) / r * d
    for g1, g2, kf, tol, off in terms.centroid:
        m = terms.masses
        c1 = (m[g1, None] * pos[g1]).sum(0) / m[g1].sum()
        c2 = (m[g2, None] * pos[g2]).sum(0) / m[g2].sum()
        d = c1 - np.asarray(off) - c2
        r = math.sqrt(float(d @ d))
        if r > tol:
            E += 0.5 * kf * (r - tol) ** 2
            g = kf * (r - tol) / r * d
            F[g1] -= (m[g1] / m[g1].sum())[:, None] * g
            F[g2] += (m[g2] / m[g2].sum())[:, None] * g
    return E, F


def constraint_clusters(constraints, n):
    """Clusters of the constraint graph in order of first appearance, each
    (atoms, [(local a, local b, d^2)]) with at most 4 atoms."""
    parent = list(range(n))

    def find(i):
        while parent[i] != i:
            parent[i] = parent[parent[i]]
            i = parent[i]
        return i

    for i, j, _ in constraints:
        parent[find(i)] = find(j)
    groups, order = {}, []
    for i, j, d in constraints:
        r = find(i)
        if r not in groups:
            groups[r] = ([], [])
            order.append(r)
        atoms, cons = groups[r]
        for a in (i, j):
            if a not in atoms:
                atoms.append(a)
        assert len(atoms) <= 4
        cons.append((atoms.index(i), atoms.index(j), d * d))
    return [groups[r] for r in order]


def shake(xref, x, inv_m, clusters, tol=1e-13, max_iter=10000):
    """SHAKE sweeps per cluster until every |d^2 - r^2| <= 2 tol d^2, in the GPU's order."""
    x = x.copy()
    for atoms, cons in clusters:
        p = x[atoms].copy()
        ref = xref[atoms]
        im = inv_m[atoms]
        for _ in range(max_iter):
            done = True
            for a, b, d2 in cons:
                r = p[a] - p[b]
                rr = ref[a] - ref[b]
                diff = d2 - float(r @ r)
                if abs(diff) > 2.0 * tol * d2:
                    done = False
                    den = 2.0 * (im[a] + im[b]) * float(r @ rr)
                    g = diff / den if den != 0.0 else 0.0
                    p[a] += g * im[a] * rr
                    p[b] -= g * im[b] * rr
            if done:
                break
        else:
            raise RuntimeError("SHAKE did not converge")
        x[atoms] = p
    return x


def langevin_step(x, v, f, inv_m, T, gamma, dt, seed, step, clusters, tol=1e-13, replica=0):
    """One leapfrog Langevin step of one replica with total force f at x; returns (x', v')."""
    a = math.exp(-gamma * dt)
    fs = dt if gamma == 0.0 else (1.0 - a) / gamma
    ns = math.sqrt(KB * T * (1.0 - a * a))
    z = normals3(len(x), step, RNG_THERMOSTAT, seed, replica)
    moving = inv_m > 0
    vn = a * v + fs * f * inv_m[:, None] + ns * np.sqrt(inv_m)[:, None] * z
    xn = x + dt * vn
    xn = shake(x, xn, inv_m, clusters, tol)
    vn = (xn - x) / dt
    vn[~moving] = 0.0
    xn[~moving] = x[~moving]
    return xn, vn


def project_velocities(x, w, inv_m, clusters, tol=1e-12, max_iter=200):
    """Remove from w its components along the constraints at x (velocity RATTLE),
    in the GPU's sweep order."""
    w = w.copy()
    for atoms, cons in clusters:
        p = x[atoms]
        u = w[atoms].copy()
        im = inv_m[atoms]
        for _ in range(max_iter):
            done = True
            for a, b, _ in cons:
                r = p[a] - p[b]
                dv = u[a] - u[b]
                r2 = float(r @ r)
                proj = float(dv @ r)
                scale = math.sqrt(r2 * (float(u[a] @ u[a]) + float(u[b] @ u[b]))) + 1e-300
                if abs(proj) > tol * scale:
                    done = False
                    g = proj / ((im[a] + im[b]) * r2)
                    u[a] -= g * im[a] * r
                    u[b] += g * im[b] * r
            if done:
                break
        w[atoms] = u
    return w


def kinetic(v, f, inv_m, dt, x=None, clusters=()):
    """Kinetic energy of the on-step velocities v + dt/2 f/m, with their
    components along the constraints at x removed, over particles with mass."""
    m = inv_m > 0
    w = np.where(m[:, None], v + 0.5 * dt * f * inv_m[:, None], 0.0)
    if clusters:
        w = project_velocities(x, w, inv_m, clusters)
    return float(0.5 * ((w[m] * w[m]).sum(1) / inv_m[m]).sum())


def velocities_at(T, inv_m, seed, replica=0, x=None, clusters=()):
    """Maxwell-Boltzmann velocities as the GPU draws them (stream 1, step 0),
    projected off the constraints at x when clusters are given."""
    z = normals3(len(inv_m), 0, RNG_VELOCITIES, seed, replica)
    v = np.sqrt(KB * T * inv_m)[:, None] * z
    if clusters:
        v = project_velocities(x, v, inv_m, clusters)
    return v
