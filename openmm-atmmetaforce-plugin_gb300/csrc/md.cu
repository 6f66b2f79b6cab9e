// Langevin dynamics driver: group-0 terms, leapfrog Langevin update, SHAKE
// clusters, kinetic energy.  One thread per term / atom / constraint cluster;
// all of it is a few percent of a step next to the ATM evaluation.
#include "md.h"

#include <sstream>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>

#include "philox.h"

namespace atm {

#define MD_CHECK(x)                                                                              \
    do {                                                                                         \
        cudaError_t e_ = (x);                                                                    \
        if (e_ != cudaSuccess) throw Error(4, std::string("CUDA error: ") + cudaGetErrorString(e_)); \
    } while (0)

struct MdDev {
    int n, R;
    const double* x;
    double* v;
    double* xn;
    const double* inv_m;
    const double* sqrt_inv_m;  // per atom, for the thermostat noise
    const int* rep_of;
    const double* f_atm;
    unsigned long long* fb;
    double* e_terms;
    const MdBond* bonds;
    const MdAngle* angles;
    const MdPosRes* posres;
    const MdCentroid* cent;
    const int* cent_idx;
    const double* cent_w;
    const MdConsGroup* cons;
    const MdSettle* settle;
    const int* free_atoms;  // atoms in no constraint unit
    int n_bonds, n_angles, n_posres, n_cent, n_cons, n_settle, n_free;
    const double* box;  // 6 per replica: ax, by, cz, bx, cx, cy (reduced box vectors)
    const int* rep_off; // R + 1
    double* ke;         // R
    int* status;
    // integrator
    double dt, vscale, fscale, noisescale, tol;
    uint32_t seed_lo, seed_hi;
    uint32_t step_lo, step_hi;
};

namespace {

__device__ __forceinline__ void fadd(unsigned long long* p, double v) {
    atomicAdd(p, (unsigned long long)__double2ll_rn(v * kFixScale));
}

__device__ __forceinline__ double fix_to_d(unsigned long long u) { return (double)(long long)u / kFixScale; }

__global__ void k_md_terms(MdDev a) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int nt = a.n_bonds + a.n_angles + a.n_posres;
    if (t >= nt) return;
    double E = 0.0;
    if (t < a.n_bonds) {
        MdBond b = a.bonds[t];
        double d[3], r2 = 0.0;
        for (int k = 0; k < 3; k++) {
            d[k] = a.x[3 * (size_t)b.j + k] - a.x[3 * (size_t)b.i + k];
            r2 += d[k] * d[k];
        }
        double r = sqrt(r2), dr = r - b.length;
        E = 0.5 * b.k * dr * dr;
        double f = r > 0.0 ? b.k * dr / r : 0.0;
        for (int k = 0; k < 3; k++) {
            fadd(a.fb + 3 * (size_t)b.i + k, f * d[k]);
            fadd(a.fb + 3 * (size_t)b.j + k, -f * d[k]);
        }
    } else if (t < a.n_bonds + a.n_angles) {
        MdAngle g = a.angles[t - a.n_bonds];
        double r1[3], r2[3];
        for (int k = 0; k < 3; k++) {
            r1[k] = a.x[3 * (size_t)g.i + k] - a.x[3 * (size_t)g.j + k];
            r2[k] = a.x[3 * (size_t)g.l + k] - a.x[3 * (size_t)g.j + k];
        }
        double cp[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2], r1[0] * r2[1] - r1[1] * r2[0]};
        double ncp = sqrt(cp[0] * cp[0] + cp[1] * cp[1] + cp[2] * cp[2]);
        double dot = r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2];
        double theta = atan2(ncp, dot);
        double dth = theta - g.angle;
        E = 0.5 * g.k * dth * dth;
        if (ncp > 0.0) {
            double dE = g.k * dth;
            double n1 = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
            double n2 = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
            // d theta / d r1 = r1 x cp / (|r1|^2 |cp|), d theta / d r2 = -r2 x cp / (|r2|^2 |cp|)
            double c1[3] = {r1[1] * cp[2] - r1[2] * cp[1], r1[2] * cp[0] - r1[0] * cp[2], r1[0] * cp[1] - r1[1] * cp[0]};
            double c2[3] = {r2[1] * cp[2] - r2[2] * cp[1], r2[2] * cp[0] - r2[0] * cp[2], r2[0] * cp[1] - r2[1] * cp[0]};
            double s1 = -dE / (n1 * ncp), s2 = dE / (n2 * ncp);
            for (int k = 0; k < 3; k++) {
                double fi = s1 * c1[k], fl = s2 * c2[k];
                fadd(a.fb + 3 * (size_t)g.i + k, fi);
                fadd(a.fb + 3 * (size_t)g.l + k, fl);
                fadd(a.fb + 3 * (size_t)g.j + k, -fi - fl);
            }
        }
    } else {
        MdPosRes p = a.posres[t - a.n_bonds - a.n_angles];
        const double* L = a.box + 6 * p.rep;
        double d[3] = {a.x[3 * (size_t)p.p] - p.x0, a.x[3 * (size_t)p.p + 1] - p.y0, a.x[3 * (size_t)p.p + 2] - p.z0};
        if (p.periodic) {
            // OpenMM's minimum image: c, then b, then a
            double k = rint(d[2] / L[2]);
            d[0] -= k * L[4];
            d[1] -= k * L[5];
            d[2] -= k * L[2];
            k = rint(d[1] / L[1]);
            d[0] -= k * L[3];
            d[1] -= k * L[1];
            d[0] -= L[0] * rint(d[0] / L[0]);
        }
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (r > p.tol) {
            double dr = r - p.tol;
            E = 0.5 * p.fc * dr * dr;
            double f = -p.fc * dr / r;
            for (int k = 0; k < 3; k++) fadd(a.fb + 3 * (size_t)p.p + k, f * d[k]);
        }
    }
    a.e_terms[t] = E;
}

// One CTA per centroid restraint; fixed-order sums.
__global__ void __launch_bounds__(128) k_md_centroid(MdDev a) {
    __shared__ double red[6][128];
    const MdCentroid c = a.cent[blockIdx.x];
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int k = threadIdx.x; k < c.g1_n; k += 128) {
        int i = a.cent_idx[c.g1_off + k];
        double w = a.cent_w[c.g1_off + k];
        for (int d = 0; d < 3; d++) s[d] += w * a.x[3 * (size_t)i + d];
    }
    for (int k = threadIdx.x; k < c.g2_n; k += 128) {
        int i = a.cent_idx[c.g2_off + k];
        double w = a.cent_w[c.g2_off + k];
        for (int d = 0; d < 3; d++) s[3 + d] += w * a.x[3 * (size_t)i + d];
    }
    for (int d = 0; d < 6; d++) red[d][threadIdx.x] = s[d];
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int d = 0; d < 6; d++) red[d][threadIdx.x] += red[d][threadIdx.x + o];
        __syncthreads();
    }
    double dv[3];
    for (int d = 0; d < 3; d++) dv[d] = red[d][0] / c.m1 - c.off[d] - red[3 + d][0] / c.m2;
    double r = sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    double E = 0.0, g = 0.0;
    if (r > c.tol) {
        double dr = r - c.tol;
        E = 0.5 * c.kf * dr * dr;
        g = c.kf * dr / r;  // dE/dc1 = g dv
    }
    if (g != 0.0) {
        for (int k = threadIdx.x; k < c.g1_n; k += 128) {
            int i = a.cent_idx[c.g1_off + k];
            double w = a.cent_w[c.g1_off + k] / c.m1;
            for (int d = 0; d < 3; d++) fadd(a.fb + 3 * (size_t)i + d, -g * w * dv[d]);
        }
        for (int k = threadIdx.x; k < c.g2_n; k += 128) {
            int i = a.cent_idx[c.g2_off + k];
            double w = a.cent_w[c.g2_off + k] / c.m2;
            for (int d = 0; d < 3; d++) fadd(a.fb + 3 * (size_t)i + d, g * w * dv[d]);
        }
    }
    if (threadIdx.x == 0) a.e_terms[a.n_bonds + a.n_angles + a.n_posres + blockIdx.x] = E;
}

// Three standard normals from one Philox block: Box-Muller in FP32 on two
// pairs of 24-bit uniforms in (0, 1).  The counter is (atom index within its
// replica, step low, step high, replica << 1 | stream), so a replica's noise does
// not depend on the other replicas of a batch.
__device__ __forceinline__ void normals3(uint32_t i, uint32_t s0, uint32_t s1, uint32_t stream, uint32_t k0,
                                         uint32_t k1, double z[3]) {
    U32x4 c = {{i, s0, s1, stream}};
    U32x4 r = philox4x32_10(c, k0, k1);
    const float inv24 = 1.0f / 16777216.0f;
    float u0 = ((float)(r.v[0] >> 8) + 0.5f) * inv24, u1 = ((float)(r.v[1] >> 8) + 0.5f) * inv24;
    float u2 = ((float)(r.v[2] >> 8) + 0.5f) * inv24, u3 = ((float)(r.v[3] >> 8) + 0.5f) * inv24;
    float a = sqrtf(-2.0f * logf(u0)), b = sqrtf(-2.0f * logf(u2));
    float s1f, c1f, s3f, c3f;
    sincospif(2.0f * u1, &s1f, &c1f);
    sincospif(2.0f * u3, &s3f, &c3f);
    z[0] = (double)(a * c1f);
    z[1] = (double)(a * s1f);
    z[2] = (double)(b * c3f);
}

// The Langevin update of atom i: the unconstrained new position xn from x, the
// previous velocity, the forces and the thermostat noise (the velocity is set
// from the constrained position afterwards, md_finish).
__device__ __forceinline__ void md_integrate(const MdDev& a, int i, double* xn) {
    double im = a.inv_m[i];
    if (im == 0.0) {
        for (int k = 0; k < 3; k++) xn[k] = a.x[3 * (size_t)i + k];
        return;
    }
    double z[3];
    const int r = a.rep_of[i];
    normals3((uint32_t)(i - a.rep_off[r]), a.step_lo, a.step_hi, ((uint32_t)r << 1) | RNG_THERMOSTAT, a.seed_lo,
             a.seed_hi, z);
    // FP64 is scarce on this part: per-atom factors once, then four fused
    // multiply-adds per component
    const double fim = a.fscale * im, nsim = a.noisescale * a.sqrt_inv_m[i];
    for (int k = 0; k < 3; k++) {
        size_t o = 3 * (size_t)i + k;
        const double f = fma((double)(long long)a.fb[o], 1.0 / kFixScale, a.f_atm[o]);
        const double v = fma(nsim, z[k], fma(fim, f, a.vscale * a.v[o]));
        xn[k] = fma(a.dt, v, a.x[o]);
    }
}

// v = (x' - x) / dt and x <- x' for atom i (massless atoms keep v = 0).
__device__ __forceinline__ void md_finish(const MdDev& a, double* x, int i, const double* xn) {
    const double inv_dt = 1.0 / a.dt;
    const bool massless = a.inv_m[i] == 0.0;
    for (int k = 0; k < 3; k++) {
        const size_t o = 3 * (size_t)i + k;
        a.v[o] = massless ? 0.0 : (xn[k] - x[o]) * inv_dt;
        x[o] = xn[k];
    }
}

// SHAKE iterations on one cluster: p (the unconstrained new positions) corrected
// along the reference (pre-step) bonds; false when they did not converge.
__device__ bool md_shake(const MdDev& a, const MdConsGroup& c, const double (*ref)[3], double (*p)[3],
                         const double* im) {
    bool done = false;
    for (int it = 0; it < 1000 && !done; it++) {
        done = true;
        for (int q = 0; q < c.nc; q++) {
            int u = c.a[q], w = c.b[q];
            double r[3], rr[3];
            for (int d = 0; d < 3; d++) {
                r[d] = p[u][d] - p[w][d];
                rr[d] = ref[u][d] - ref[w][d];
            }
            double diff = c.d2[q] - (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            if (fabs(diff) > 2.0 * a.tol * c.d2[q]) {
                done = false;
                double den = 2.0 * (im[u] + im[w]) * (r[0] * rr[0] + r[1] * rr[1] + r[2] * rr[2]);
                double gq = den != 0.0 ? diff / den : 0.0;
                for (int d = 0; d < 3; d++) {
                    p[u][d] += gq * im[u] * rr[d];
                    p[w][d] -= gq * im[w] * rr[d];
                }
            }
        }
    }
    return done;
}

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// SETTLE: closed-form solution of the three constraints of a rigid water, the
// displacements lying in the plane of the reference (pre-step) geometry.  The
// frame: Z normal to the old triangle, X perpendicular to the new O position
// (relative to the new centre of mass) and to Z, Y = Z x X.  In that frame the
// constrained triangle is rotated by phi (about X), psi (about Y) to match the
// new out-of-plane coordinates, then by theta (about Z) so that the in-plane
// displacements are along the old bonds.

// SETTLE on one water: a0, b0, c0 the old positions of O, H1, H2; a1, b1, c1
// their unconstrained new positions, replaced by the constrained ones; false (a1,
// b1, c1 kept) when the displacement is too large for the closed form.
__device__ bool md_settle(const MdSettle& S, const double* a0, const double* b0, const double* c0, double* a1,
                          double* b1, double* c1) {
    double com[3], xa1[3], xb1[3], xc1[3], xb0[3], xc0[3];
    for (int d = 0; d < 3; d++) {
        com[d] = S.wo * a1[d] + S.wh * (b1[d] + c1[d]);
        xa1[d] = a1[d] - com[d];
        xb1[d] = b1[d] - com[d];
        xc1[d] = c1[d] - com[d];
        xb0[d] = b0[d] - a0[d];
        xc0[d] = c0[d] - a0[d];
    }
    double X[3], Y[3], Z[3];
    cross3(xb0, xc0, Z);
    cross3(xa1, Z, X);
    cross3(Z, X, Y);
    double nx = rsqrt(dot3(X, X)), ny = rsqrt(dot3(Y, Y)), nz = rsqrt(dot3(Z, Z));
    for (int d = 0; d < 3; d++) {
        X[d] *= nx;
        Y[d] *= ny;
        Z[d] *= nz;
    }
    const double xb0d = dot3(xb0, X), yb0d = dot3(xb0, Y);
    const double xc0d = dot3(xc0, X), yc0d = dot3(xc0, Y);
    const double za1d = dot3(xa1, Z);
    const double xb1d = dot3(xb1, X), yb1d = dot3(xb1, Y), zb1d = dot3(xb1, Z);
    const double xc1d = dot3(xc1, X), yc1d = dot3(xc1, Y), zc1d = dot3(xc1, Z);
    const double sinphi = za1d / S.ra;
    const double cosphi = sqrt(1.0 - sinphi * sinphi);
    const double sinpsi = (zb1d - zc1d) / (2.0 * S.rc * cosphi);
    const double cospsi = sqrt(1.0 - sinpsi * sinpsi);
    const double ya2d = S.ra * cosphi;
    const double xb2d = -S.rc * cospsi;
    const double t1 = -S.rb * cosphi, t2 = S.rc * sinpsi * sinphi;
    const double yb2d = t1 - t2, yc2d = t1 + t2;
    const double alpha = xb2d * (xb0d - xc0d) + yb0d * yb2d + yc0d * yc2d;
    const double beta = xb2d * (yc0d - yb0d) + xb0d * yb2d + xc0d * yc2d;
    const double gamma = xb0d * yb1d - xb1d * yb0d + xc0d * yc1d - xc1d * yc0d;
    const double al2be2 = alpha * alpha + beta * beta;
    const double sinthe = (alpha * gamma - beta * sqrt(al2be2 - gamma * gamma)) / al2be2;
    const double costhe = sqrt(1.0 - sinthe * sinthe);
    const double pa[3] = {-ya2d * sinthe, ya2d * costhe, za1d};
    const double pb[3] = {xb2d * costhe - yb2d * sinthe, xb2d * sinthe + yb2d * costhe, zb1d};
    const double pc[3] = {-xb2d * costhe - yc2d * sinthe, -xb2d * sinthe + yc2d * costhe, zc1d};
    double ra3[3], rb3[3], rc3[3];
    bool ok = true;
    for (int d = 0; d < 3; d++) {
        ra3[d] = com[d] + pa[0] * X[d] + pa[1] * Y[d] + pa[2] * Z[d];
        rb3[d] = com[d] + pb[0] * X[d] + pb[1] * Y[d] + pb[2] * Z[d];
        rc3[d] = com[d] + pc[0] * X[d] + pc[1] * Y[d] + pc[2] * Z[d];
        ok = ok && isfinite(ra3[d]) && isfinite(rb3[d]) && isfinite(rc3[d]);
    }
    if (!ok) return false;  // displacement too large for the closed form: leave the water
    for (int d = 0; d < 3; d++) {
        a1[d] = ra3[d];
        b1[d] = rb3[d];
        c1[d] = rc3[d];
    }
    return true;
}

// One step's update, one thread per unit: a rigid water (the Langevin update of
// its three atoms, SETTLE, the velocities from the constrained positions), a SHAKE
// cluster (likewise), or an atom in no constraint; all in registers, one pass over
// the state.  A failed constraint counts in the status and leaves its atoms at
// their unconstrained positions.
__global__ void k_md_update(MdDev a, double* x) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < a.n_settle) {
        const MdSettle S = a.settle[u];
        const int at[3] = {S.o, S.h1, S.h2};
        double x0[3][3], x1[3][3];
        for (int k = 0; k < 3; k++) {
            for (int d = 0; d < 3; d++) x0[k][d] = a.x[3 * (size_t)at[k] + d];
            md_integrate(a, at[k], x1[k]);
        }
        if (!md_settle(S, x0[0], x0[1], x0[2], x1[0], x1[1], x1[2])) atomicAdd(a.status, 1);
        for (int k = 0; k < 3; k++) md_finish(a, x, at[k], x1[k]);
        return;
    }
    const int g = u - a.n_settle;
    if (g < a.n_cons) {
        const MdConsGroup& c = a.cons[g];
        double ref[kConsAtoms][3], p[kConsAtoms][3], im[kConsAtoms];
        int na = 0;
        for (int k = 0; k < kConsAtoms; k++) {
            const int i = c.atom[k];
            if (i < 0) break;
            na = k + 1;
            im[k] = a.inv_m[i];
            for (int d = 0; d < 3; d++) ref[k][d] = a.x[3 * (size_t)i + d];
            md_integrate(a, i, p[k]);
        }
        if (!md_shake(a, c, ref, p, im)) atomicAdd(a.status, 1);
        for (int k = 0; k < na; k++) md_finish(a, x, c.atom[k], p[k]);
        return;
    }
    const int f = g - a.n_cons;
    if (f < a.n_free) {
        const int i = a.free_atoms[f];
        double xn[3];
        md_integrate(a, i, xn);
        md_finish(a, x, i, xn);
    }
}


// w = v + (dt/2) f/m: the leapfrog estimate of the on-step velocities.
__global__ void k_md_shift(MdDev a, double* w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double im = a.inv_m[i];
    for (int k = 0; k < 3; k++) {
        size_t o = 3 * (size_t)i + k;
        w[o] = im == 0.0 ? 0.0 : a.v[o] + 0.5 * a.dt * (a.f_atm[o] + fix_to_d(a.fb[o])) * im;
    }
}

// Removes from w the components along the constraints at positions x (the
// velocity half of RATTLE): Gauss-Seidel sweeps over a cluster's constraints
// until every relative velocity along a constraint is below 1e-12 of the
// velocities.  Items: the SHAKE clusters, then the SETTLE waters.
__global__ void k_md_vproject(MdDev a, double* w) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.n_cons + a.n_settle) return;
    int atoms[kConsAtoms] = {-1, -1, -1, -1};
    int ca[kConsMax], cb[kConsMax], nc;
    if (g < a.n_cons) {
        const MdConsGroup& c = a.cons[g];
        for (int k = 0; k < kConsAtoms; k++) atoms[k] = c.atom[k];
        nc = c.nc;
        for (int q = 0; q < nc; q++) {
            ca[q] = c.a[q];
            cb[q] = c.b[q];
        }
    } else {
        const MdSettle& S = a.settle[g - a.n_cons];
        atoms[0] = S.o;
        atoms[1] = S.h1;
        atoms[2] = S.h2;
        nc = 3;
        ca[0] = 0; cb[0] = 1;
        ca[1] = 0; cb[1] = 2;
        ca[2] = 1; cb[2] = 2;
    }
    double p[kConsAtoms][3], u[kConsAtoms][3], im[kConsAtoms];
    for (int k = 0; k < kConsAtoms; k++) {
        int i = atoms[k] < 0 ? atoms[0] : atoms[k];
        im[k] = atoms[k] < 0 ? 0.0 : a.inv_m[i];
        for (int d = 0; d < 3; d++) {
            p[k][d] = a.x[3 * (size_t)i + d];
            u[k][d] = w[3 * (size_t)i + d];
        }
    }
    bool done = false;
    for (int it = 0; it < 200 && !done; it++) {
        done = true;
        for (int q = 0; q < nc; q++) {
            int s = ca[q], t = cb[q];
            double r[3], dv[3];
            for (int d = 0; d < 3; d++) {
                r[d] = p[s][d] - p[t][d];
                dv[d] = u[s][d] - u[t][d];
            }
            double r2 = dot3(r, r), proj = dot3(dv, r);
            double scale = sqrt(r2 * (dot3(u[s], u[s]) + dot3(u[t], u[t]))) + 1e-300;
            if (fabs(proj) > 1e-12 * scale) {
                done = false;
                double gq = proj / ((im[s] + im[t]) * r2);
                for (int d = 0; d < 3; d++) {
                    u[s][d] -= gq * im[s] * r[d];
                    u[t][d] += gq * im[t] * r[d];
                }
            }
        }
    }
    for (int k = 0; k < kConsAtoms; k++)
        if (atoms[k] >= 0)
            for (int d = 0; d < 3; d++) w[3 * (size_t)atoms[k] + d] = u[k][d];
}

// Kinetic energy per replica of the velocities w; one CTA per replica.
__global__ void __launch_bounds__(256) k_md_kinetic(MdDev a, const double* w) {
    __shared__ double red[256];
    int r = blockIdx.x;
    double s = 0.0;
    for (int i = a.rep_off[r] + threadIdx.x; i < a.rep_off[r + 1]; i += 256) {
        double im = a.inv_m[i];
        if (im == 0.0) continue;
        const double* v = w + 3 * (size_t)i;
        s += 0.5 * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / im;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.ke[r] = red[0];
}

__global__ void k_md_velocities(MdDev a, double kT, uint32_t k0, uint32_t k1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    double im = a.inv_m[i];
    double z[3];
    const int r = a.rep_of[i];
    normals3((uint32_t)(i - a.rep_off[r]), 0u, 0u, ((uint32_t)r << 1) | RNG_VELOCITIES, k0, k1, z);
    double s = sqrt(kT * im);
    for (int k = 0; k < 3; k++) a.v[3 * (size_t)i + k] = s * z[k];
}

template <typename T>
T* md_alloc(std::vector<void*>& list, size_t n) {
    void* p = nullptr;
    MD_CHECK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    list.push_back(p);
    return (T*)p;
}

template <typename T>
T* md_upload(std::vector<void*>& list, const std::vector<T>& h) {
    T* p = md_alloc<T>(list, h.size());
    if (!h.empty()) MD_CHECK(cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return p;
}

}  // namespace

// ---------------------------------------------------------------------------

MDDriver::MDDriver(const std::vector<const System*>& systems, int device, bool full_mode, const MdOptions& opt)
    : opt_(opt), dev_(device) {
    if (systems.empty()) throw Error(1, "No replicas");
    std::vector<ReplicaSpec> specs;
    for (auto* s : systems) specs.push_back(spec_from_system(*s));
    eng_.reset(new Engine(specs, device, full_mode, false));
    R_ = eng_->replicas();
    n_ = eng_->total_atoms();
    for (int r = 0; r < R_; r++) in_off_.push_back(eng_->in_offset(r));
    MD_CHECK(cudaSetDevice(dev_));
    MD_CHECK(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    MD_CHECK(cudaStreamCreateWithFlags(&s_terms_, cudaStreamNonBlocking));
    MD_CHECK(cudaEventCreateWithFlags(&ev_x_, cudaEventDisableTiming));
    MD_CHECK(cudaEventCreateWithFlags(&ev_terms_, cudaEventDisableTiming));
    upload_terms(systems);
    update_beta();
    if (opt_.list_skin >= 0.0) {
        // no larger than the boxes allow (periodic boxes of at least 2 (cutoff + skin))
        double skin = std::min(opt_.list_skin, 0.5);
        for (auto* sys : systems) {
            const ReplicaSpec sp = spec_from_system(*sys);
            if (sp.method == NonbondedForce::CutoffPeriodic || sp.method == NonbondedForce::PME)
                for (int a = 0; a < 3; a++) skin = std::min(skin, 0.5 * sp.box[a] - sp.cutoff);
        }
        eng_->set_list_skin(std::max(0.0, skin));
        tuned_ = true;
    }
    if (opt_.check_interval < 1) throw Error(1, "The list check interval must be at least one step");
    // re-sorts are decided at the checks
    if (opt_.reorder_interval > 0) opt_.check_interval = std::min(opt_.check_interval, opt_.reorder_interval);
}

MDDriver::~MDDriver() {
    cudaSetDevice(dev_);
    if (rec_res_) cudaFree(rec_res_);
    if (rec_mat_) cudaFree(rec_mat_);
    for (void* p : allocs_) cudaFree(p);
    if (s_) cudaStreamDestroy(s_);
    if (s_terms_) cudaStreamDestroy(s_terms_);
    if (ev_x_) cudaEventDestroy(ev_x_);
    if (ev_terms_) cudaEventDestroy(ev_terms_);
}

void MDDriver::upload_terms(const std::vector<const System*>& systems) {
    std::vector<double> inv_m(n_);
    std::vector<int> rep_of(n_);
    std::vector<MdBond> bonds;
    std::vector<MdAngle> angles;
    std::vector<MdPosRes> posres;
    std::vector<MdCentroid> cent;
    std::vector<int> cent_idx;
    std::vector<double> cent_w;
    std::vector<MdConsGroup> cons;
    std::vector<double> box(6 * (size_t)R_);
    std::vector<int> rep_off(R_ + 1);
    dof_.assign(R_, 0);
    std::vector<int> bond_rep, ang_rep, pos_rep, cent_rep;
    for (int r = 0; r < R_; r++) {
        const System& S = *systems[r];
        const int n = eng_->atoms(r), o = in_off_[r];
        rep_off[r] = o;
        if ((int)S.masses.size() != n) throw Error(9, "System particle count differs from the NonbondedForce's");
        for (int k = 0; k < 3; k++) {
            box[6 * r + k] = eng_->box(r)[k];
            box[6 * r + 3 + k] = eng_->tilt(r)[k];
        }
        int moving = 0;
        for (int i = 0; i < n; i++) {
            inv_m[o + i] = S.masses[i] > 0.0 ? 1.0 / S.masses[i] : 0.0;
            rep_of[o + i] = r;
            moving += S.masses[i] > 0.0;
        }
        auto chk = [&](int i) {
            if (i < 0 || i >= n) throw Error(2, "Particle index out of range in a bonded term");
            return o + i;
        };
        for (const Bond& b : S.bonds) {
            bonds.push_back({chk(b.i), chk(b.j), r, 0, b.length, b.k});
            bond_rep.push_back(r);
        }
        for (const Angle& g : S.angles) {
            angles.push_back({chk(g.i), chk(g.j), chk(g.l), r, g.angle, g.k});
            ang_rep.push_back(r);
        }
        for (const PositionRestraint& p : S.position_restraints) {
            posres.push_back({chk(p.particle), r, S.position_restraints_periodic ? 1 : 0, 0, p.x0, p.y0, p.z0, p.fc,
                              p.tol});
            pos_rep.push_back(r);
        }
        for (const CentroidRestraint& c : S.centroid_restraints) {
            if (c.g1.empty() || c.g2.empty()) throw Error(1, "Empty centroid group");
            MdCentroid d{};
            d.rep = r;
            d.kf = c.kf;
            d.tol = c.tol;
            for (int k = 0; k < 3; k++) d.off[k] = c.offset[k];
            d.g1_off = (int)cent_idx.size();
            d.g1_n = (int)c.g1.size();
            for (int i : c.g1) {
                cent_idx.push_back(chk(i));
                cent_w.push_back(S.masses[i]);
                d.m1 += S.masses[i];
            }
            d.g2_off = (int)cent_idx.size();
            d.g2_n = (int)c.g2.size();
            for (int i : c.g2) {
                cent_idx.push_back(chk(i));
                cent_w.push_back(S.masses[i]);
                d.m2 += S.masses[i];
            }
            if (!(d.m1 > 0.0) || !(d.m2 > 0.0)) throw Error(1, "Centroid group without mass");
            cent.push_back(d);
            cent_rep.push_back(r);
        }
        // constraint clusters: connected components of the constraint graph
        std::vector<int> parent(n);
        std::iota(parent.begin(), parent.end(), 0);
        std::function<int(int)> find = [&](int i) { return parent[i] == i ? i : parent[i] = find(parent[i]); };
        for (const Constraint& c : S.constraints) {
            chk(c.i);
            chk(c.j);
            if (c.i == c.j || !(c.distance > 0.0)) throw Error(1, "Invalid constraint");
            if (S.masses[c.i] <= 0.0 && S.masses[c.j] <= 0.0) throw Error(1, "Constraint between two massless particles");
            parent[find(c.i)] = find(c.j);
        }
        std::map<int, int> root_group;
        for (const Constraint& c : S.constraints) {
            int root = find(c.i);
            auto it = root_group.find(root);
            if (it == root_group.end()) {
                MdConsGroup g{};
                for (int k = 0; k < kConsAtoms; k++) g.atom[k] = -1;
                it = root_group.emplace(root, (int)cons.size()).first;
                cons.push_back(g);
            }
            MdConsGroup& g = cons[it->second];
            auto slot = [&](int i) {
                for (int k = 0; k < kConsAtoms; k++) {
                    if (g.atom[k] == o + i) return k;
                    if (g.atom[k] < 0) {
                        g.atom[k] = o + i;
                        return k;
                    }
                }
                throw Error(5, "Constraint cluster of more than 4 particles (SHAKE clusters hold at most 4)");
            };
            if (g.nc >= kConsMax) throw Error(5, "Constraint cluster of more than 6 constraints");
            g.a[g.nc] = slot(c.i);
            g.b[g.nc] = slot(c.j);
            g.d2[g.nc] = c.distance * c.distance;
            g.nc++;
        }
        dof_[r] = 3 * moving - (int)S.constraints.size();
    }
    // rigid waters go to SETTLE, every other cluster to SHAKE
    std::vector<MdConsGroup> shake_groups;
    std::vector<MdSettle> settle;
    for (const MdConsGroup& g : cons) {
        bool water = false;
        if (g.nc == 3 && g.atom[2] >= 0 && g.atom[3] < 0) {
            for (int o = 0; o < 3 && !water; o++) {
                // o bonded to both others with one length, the other two joined by the third
                int idx[2], k = 0;
                double dOH = -1.0, dHH = -1.0;
                bool okk = true;
                for (int q = 0; q < 3; q++) {
                    double d = std::sqrt(g.d2[q]);
                    if (g.a[q] == o || g.b[q] == o) {
                        int other = g.a[q] == o ? g.b[q] : g.a[q];
                        if (k < 2) idx[k++] = other;
                        if (dOH < 0) dOH = d;
                        else if (std::fabs(d - dOH) > 1e-12 * dOH) okk = false;
                    } else {
                        dHH = d;
                    }
                }
                if (!okk || k != 2 || dHH <= 0.0 || dHH >= 2.0 * dOH) continue;
                int ao = g.atom[o], a1 = g.atom[idx[0]], a2 = g.atom[idx[1]];
                double mo = 1.0 / inv_m[ao], mh = 1.0 / inv_m[a1];
                if (inv_m[ao] == 0.0 || inv_m[a1] == 0.0 || inv_m[a1] != inv_m[a2]) continue;
                MdSettle w{};
                w.o = ao;
                w.h1 = a1;
                w.h2 = a2;
                double t = mo + 2.0 * mh;
                w.wo = mo / t;
                w.wh = mh / t;
                w.rc = 0.5 * dHH;
                double h = std::sqrt(dOH * dOH - w.rc * w.rc);
                w.ra = 2.0 * mh * h / t;
                w.rb = h - w.ra;
                settle.push_back(w);
                water = true;
            }
        }
        if (!water) shake_groups.push_back(g);
    }
    cons.swap(shake_groups);
    std::vector<int> free_atoms;
    {
        std::vector<char> in_unit(n_, 0);
        for (const MdSettle& w : settle) in_unit[w.o] = in_unit[w.h1] = in_unit[w.h2] = 1;
        for (const MdConsGroup& g : cons)
            for (int k = 0; k < kConsAtoms; k++)
                if (g.atom[k] >= 0) in_unit[g.atom[k]] = 1;
        for (int i = 0; i < n_; i++)
            if (!in_unit[i]) free_atoms.push_back(i);
    }
    n_free_ = (int)free_atoms.size();
    rep_off[R_] = n_;
    n_bonds_ = (int)bonds.size();
    n_angles_ = (int)angles.size();
    n_posres_ = (int)posres.size();
    n_cent_ = (int)cent.size();
    n_cons_ = (int)cons.size();
    n_settle_ = (int)settle.size();
    term_rep_.clear();
    for (auto v : {&bond_rep, &ang_rep, &pos_rep, &cent_rep}) term_rep_.insert(term_rep_.end(), v->begin(), v->end());

    x_ = md_alloc<double>(allocs_, 3 * (size_t)n_);
    eng_->set_position_source(x_);  // every evaluation reads the MD positions in place
    v_ = md_alloc<double>(allocs_, 3 * (size_t)n_);
    xn_ = md_alloc<double>(allocs_, 3 * (size_t)n_);
    MD_CHECK(cudaMemset(v_, 0, sizeof(double) * 3 * (size_t)n_));
    inv_m_ = md_upload(allocs_, inv_m);
    {
        std::vector<double> sq(n_);
        for (int i = 0; i < n_; i++) sq[i] = std::sqrt(inv_m[i]);
        sqrt_inv_m_ = md_upload(allocs_, sq);
    }
    rep_of_ = md_upload(allocs_, rep_of);
    fb_ = md_alloc<unsigned long long>(allocs_, 3 * (size_t)n_);
    MD_CHECK(cudaMemset(fb_, 0, sizeof(unsigned long long) * 3 * (size_t)n_));
    e_terms_ = md_alloc<double>(allocs_, term_rep_.size());
    status_ = md_alloc<int>(allocs_, 1);
    MD_CHECK(cudaMemset(status_, 0, sizeof(int)));
    bonds_ = md_upload(allocs_, bonds);
    angles_ = md_upload(allocs_, angles);
    posres_ = md_upload(allocs_, posres);
    cent_ = md_upload(allocs_, cent);
    cent_idx_ = md_upload(allocs_, cent_idx);
    cent_w_ = md_upload(allocs_, cent_w);
    cons_ = md_upload(allocs_, cons);
    settle_ = md_upload(allocs_, settle);
    free_ = md_upload(allocs_, free_atoms);
    box_d_ = md_upload(allocs_, box);
    rep_off_d_ = md_upload(allocs_, rep_off);
    ke_d_ = md_alloc<double>(allocs_, R_);
    x_snap_ = md_alloc<double>(allocs_, 3 * (size_t)n_);
    v_snap_ = md_alloc<double>(allocs_, 3 * (size_t)n_);
}

MdDev MDDriver::dev_args() const {
    MdDev a{};
    const MdOptions& o = opt_;
    a.n = n_;
    a.R = R_;
    a.x = x_;
    a.v = v_;
    a.xn = xn_;
    a.inv_m = inv_m_;
    a.sqrt_inv_m = sqrt_inv_m_;
    a.rep_of = rep_of_;
    a.f_atm = eng_->forces_device();
    a.fb = fb_;
    a.e_terms = e_terms_;
    a.bonds = bonds_;
    a.angles = angles_;
    a.posres = posres_;
    a.cent = cent_;
    a.cent_idx = cent_idx_;
    a.cent_w = cent_w_;
    a.cons = cons_;
    a.settle = settle_;
    a.free_atoms = free_;
    a.n_free = n_free_;
    a.n_bonds = n_bonds_;
    a.n_angles = n_angles_;
    a.n_posres = n_posres_;
    a.n_cent = n_cent_;
    a.n_cons = n_cons_;
    a.n_settle = n_settle_;
    a.box = box_d_;
    a.rep_off = rep_off_d_;
    a.ke = ke_d_;
    a.status = status_;
    a.dt = o.step_size;
    a.vscale = std::exp(-o.step_size * o.friction);
    a.fscale = o.friction == 0.0 ? o.step_size : (1.0 - a.vscale) / o.friction;
    a.noisescale = std::sqrt(kBoltz * o.temperature * (1.0 - a.vscale * a.vscale));
    a.tol = o.constraint_tol;
    a.seed_lo = (uint32_t)o.seed;
    a.seed_hi = (uint32_t)(o.seed >> 32);
    a.step_lo = (uint32_t)step_;
    a.step_hi = (uint32_t)((unsigned long long)step_ >> 32);
    return a;
}

void MDDriver::set_positions(const double* pos) {
    MD_CHECK(cudaSetDevice(dev_));
    MD_CHECK(cudaMemcpy(x_, pos, sizeof(double) * 3 * (size_t)n_, cudaMemcpyHostToDevice));
    have_positions_ = true;
    forces_valid_ = false;
}

void MDDriver::set_velocities(const double* vel) {
    MD_CHECK(cudaSetDevice(dev_));
    MD_CHECK(cudaMemcpy(v_, vel, sizeof(double) * 3 * (size_t)n_, cudaMemcpyHostToDevice));
}

void MDDriver::set_velocities_to_temperature(double T, uint64_t seed) {
    MD_CHECK(cudaSetDevice(dev_));
    MdDev a = dev_args();
    k_md_velocities<<<(n_ + 255) / 256, 256, 0, s_>>>(a, kBoltz * T, (uint32_t)seed, (uint32_t)(seed >> 32));
    // no velocity along a constraint (Context::setVelocitiesToTemperature applies the velocity constraints)
    if (have_positions_ && n_cons_ + n_settle_ > 0)
        k_md_vproject<<<(n_cons_ + n_settle_ + 127) / 128, 128, 0, s_>>>(a, v_);
    MD_CHECK(cudaGetLastError());
    MD_CHECK(cudaStreamSynchronize(s_));
}

void MDDriver::set_param(int r, int which, double v) {
    eng_->set_param(r, which, v);
    forces_valid_ = false;
}

void MDDriver::set_integrator(double T, double friction, double dt) {
    if (!(dt > 0.0) || friction < 0.0 || T < 0.0) throw Error(1, "Invalid integrator parameters");
    opt_.temperature = T;
    opt_.friction = friction;
    opt_.step_size = dt;
    update_beta();
}

void MDDriver::update_beta() {
    // the reduced-energy matrix at the integrator's temperature (beta = 1 at T = 0)
    eng_->set_beta(opt_.temperature > 0.0 ? 1.0 / (kBoltz * opt_.temperature) : 1.0);
    forces_valid_ = false;
}

void MDDriver::set_recording(int interval, int capacity) {
    if (interval < 0 || (interval > 0 && capacity < 1)) throw Error(1, "Invalid recording interval or capacity");
    MD_CHECK(cudaSetDevice(dev_));
    if (rec_res_) cudaFree(rec_res_);
    if (rec_mat_) cudaFree(rec_mat_);
    rec_res_ = rec_mat_ = nullptr;
    rec_interval_ = interval;
    rec_cap_ = interval > 0 ? capacity : 0;
    rec_count_ = 0;
    rec_last_step_ = -1;
    rec_steps_.assign(rec_cap_, 0);
    if (rec_cap_ > 0) {
        MD_CHECK(cudaMalloc(&rec_res_, sizeof(double) * (size_t)rec_cap_ * R_ * NUM_RES));
        MD_CHECK(cudaMalloc(&rec_mat_, sizeof(double) * (size_t)rec_cap_ * R_ * R_));
    }
}

// Device-to-device copies of the current evaluation into the ring (no host wait).
void MDDriver::record_step() {
    if (rec_interval_ <= 0 || step_ % rec_interval_ != 0 || step_ == rec_last_step_) return;
    const int slot = (int)(rec_count_ % rec_cap_);
    MD_CHECK(cudaMemcpyAsync(rec_res_ + (size_t)slot * R_ * NUM_RES, eng_->results_device(),
                             sizeof(double) * R_ * NUM_RES, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaMemcpyAsync(rec_mat_ + (size_t)slot * R_ * R_, eng_->matrix_device(), sizeof(double) * R_ * R_,
                             cudaMemcpyDeviceToDevice, s_));
    rec_steps_[slot] = step_;
    rec_count_++;
    rec_last_step_ = step_;
}

int MDDriver::get_records(long long* steps, double* results, double* matrices, int max) {
    MD_CHECK(cudaSetDevice(dev_));
    MD_CHECK(cudaStreamSynchronize(s_));
    const long long kept = std::min<long long>(rec_count_, rec_cap_);
    const int n = (int)std::min<long long>(kept, std::max(0, max));
    const long long first = rec_count_ - kept;  // oldest kept record
    for (int k = 0; k < n; k++) {
        const int slot = (int)((first + k) % rec_cap_);
        if (steps) steps[k] = rec_steps_[slot];
        if (results)
            MD_CHECK(cudaMemcpy(results + (size_t)k * R_ * NUM_RES, rec_res_ + (size_t)slot * R_ * NUM_RES,
                                sizeof(double) * R_ * NUM_RES, cudaMemcpyDeviceToHost));
        if (matrices)
            MD_CHECK(cudaMemcpy(matrices + (size_t)k * R_ * R_, rec_mat_ + (size_t)slot * R_ * R_,
                                sizeof(double) * R_ * R_, cudaMemcpyDeviceToHost));
    }
    rec_count_ = 0;
    return n;
}

// The group-0 terms and the ATM evaluation at the current positions.  sync: wait
// for the evaluation and grow the list capacities if a build overflowed (then
// evaluate again); otherwise the evaluation is only enqueued.
void MDDriver::compute_forces(bool sync) {
    if (!have_positions_) throw Error(3, "Positions have not been set");
    MD_CHECK(cudaSetDevice(dev_));
    // the group-0 terms on their own stream, beside the ATM evaluation (after the
    // positions are final; joined before anything on s_ reads their forces)
    MD_CHECK(cudaEventRecord(ev_x_, s_));
    MD_CHECK(cudaStreamWaitEvent(s_terms_, ev_x_, 0));
    MD_CHECK(cudaMemsetAsync(fb_, 0, sizeof(unsigned long long) * 3 * (size_t)n_, s_terms_));
    {
        MdDev a = dev_args();
        int nt = n_bonds_ + n_angles_ + n_posres_;
        if (nt > 0) k_md_terms<<<(nt + 127) / 128, 128, 0, s_terms_>>>(a);
        if (n_cent_ > 0) k_md_centroid<<<n_cent_, 128, 0, s_terms_>>>(a);
        MD_CHECK(cudaGetLastError());
    }
    MD_CHECK(cudaEventRecord(ev_terms_, s_terms_));
    if (sync) eng_->run_device(x_, s_);  // synchronises and grows capacities as needed
    else eng_->launch_device(x_, s_);
    MD_CHECK(cudaStreamWaitEvent(s_, ev_terms_, 0));
    forces_valid_ = true;
}

void MDDriver::snapshot() {
    MD_CHECK(cudaMemcpyAsync(x_snap_, x_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaMemcpyAsync(v_snap_, v_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToDevice, s_));
    step_snap_ = step_;
    rec_count_snap_ = rec_count_;
    rec_last_snap_ = rec_last_step_;
}

void MDDriver::restore() {
    MD_CHECK(cudaMemcpyAsync(x_, x_snap_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaMemcpyAsync(v_, v_snap_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToDevice, s_));
    step_ = step_snap_;
    rec_count_ = rec_count_snap_;
    rec_last_step_ = rec_last_snap_;
    forces_valid_ = false;
}

bool MDDriver::check_lists() {
    MD_CHECK(cudaStreamSynchronize(s_));
    if (eng_->poll_overflow()) return true;
    if (opt_.fail_check > 0 && ++checks_ == opt_.fail_check) {
        // the test hook: handled as an overflow (the lists are built again)
        eng_->force_build();
        return true;
    }
    // re-sort when the pair-tile count shows the atom order has decayed
    int tiles = 0;
    eng_->stats(&tiles, nullptr, nullptr);
    // the baseline belongs to one list cutoff: a larger skin lists more tiles
    if (base_skin_ != eng_->list_skin()) {
        base_skin_ = eng_->list_skin();
        base_tiles_ = 0;
    }
    if (base_tiles_ == 0) base_tiles_ = tiles;
    bool due = opt_.reorder_interval > 0 ? step_ - last_reorder_step_ >= opt_.reorder_interval
                                         : tiles > base_tiles_ + base_tiles_ / 5;
    if (due && step_ > last_reorder_step_) {
        // the layout is rebuilt at the next evaluation
        eng_->reorder_from_device(x_, s_);
        reorders_++;
        base_tiles_ = 0;
        last_reorder_step_ = step_;
        forces_valid_ = false;
    }
    return false;
}

void MDDriver::step(int nsteps) {
    if (nsteps < 0) throw Error(1, "Negative step count");
    MD_CHECK(cudaSetDevice(dev_));
    if (nsteps == 0) return;
    if (!tuned_) autotune(20);
    if (!forces_valid_) compute_forces(true);
    snapshot();
    int since = 0;
    for (int k = 0; k < nsteps;) {
        if (!forces_valid_) compute_forces(false);
        record_step();
        MdDev a = dev_args();
        const int units = n_settle_ + n_cons_ + n_free_;
        if (units > 0) k_md_update<<<(units + 127) / 128, 128, 0, s_>>>(a, x_);
        MD_CHECK(cudaGetLastError());
        step_++;
        k++;
        since++;
        forces_valid_ = false;
        if (since >= opt_.check_interval || k == nsteps) {
            // the forces of the next step first: their list build is checked too
            compute_forces(false);
            if (check_lists()) {
                // an overflowed build: back to the snapshot, with grown capacities
                const long long redo = step_ - step_snap_;
                redos_++;
                restore();
                k -= (int)redo;
                compute_forces(true);
            }
            snapshot();
            since = 0;
        }
    }
    int failed = 0;
    MD_CHECK(cudaMemcpyAsync(&failed, status_, sizeof(int), cudaMemcpyDeviceToHost, s_));
    MD_CHECK(cudaStreamSynchronize(s_));
    if (failed) {
        MD_CHECK(cudaMemset(status_, 0, sizeof(int)));
        throw Error(10, "Constraints failed (SHAKE did not converge or SETTLE had no solution) in " +
                            std::to_string(failed) + " cluster-steps");
    }
}

std::string MDDriver::autotune(int trials) {
    if (trials < 1) throw Error(1, "trials must be positive");
    if (!have_positions_) throw Error(3, "Positions have not been set");
    MD_CHECK(cudaSetDevice(dev_));
    tuned_ = true;  // the steps below do not tune again
    std::ostringstream rep;
    if (!forces_valid_) compute_forces(true);
    rep << eng_->autotune(3, true);
    // the state every trial starts from, and that the simulation continues from
    double *xt = nullptr, *vt = nullptr;
    const size_t bytes = sizeof(double) * 3 * (size_t)n_;
    MD_CHECK(cudaMalloc(&xt, bytes));
    MD_CHECK(cudaMalloc(&vt, bytes));
    MD_CHECK(cudaMemcpyAsync(xt, x_, bytes, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaMemcpyAsync(vt, v_, bytes, cudaMemcpyDeviceToDevice, s_));
    const long long s0 = step_, r0 = rec_count_, l0 = rec_last_step_;
    const int rec = rec_interval_;
    rec_interval_ = 0;
    double best_ms = 1e30, best = eng_->list_skin();
    const double cands[] = {0.0, 0.05, 0.1, 0.15, 0.2};
    cudaEvent_t e0, e1;
    MD_CHECK(cudaEventCreate(&e0));
    MD_CHECK(cudaEventCreate(&e1));
    for (double skin : cands) {
        try {
            eng_->set_list_skin(skin);
        } catch (const Error&) {
            continue;  // the box is too small for this skin
        }
        MD_CHECK(cudaMemcpyAsync(x_, xt, bytes, cudaMemcpyDeviceToDevice, s_));
        MD_CHECK(cudaMemcpyAsync(v_, vt, bytes, cudaMemcpyDeviceToDevice, s_));
        step_ = s0;
        forces_valid_ = false;
        step(std::max(2, trials / 4));  // graph capture and capacities
        MD_CHECK(cudaEventRecord(e0, s_));
        step(trials);
        MD_CHECK(cudaEventRecord(e1, s_));
        MD_CHECK(cudaEventSynchronize(e1));
        float ms = 0.f;
        MD_CHECK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= trials;
        rep << "list skin " << skin << " nm: " << ms << " ms/step\n";
        if (ms < best_ms) {
            best_ms = ms;
            best = skin;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    eng_->set_list_skin(best);
    MD_CHECK(cudaMemcpyAsync(x_, xt, bytes, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaMemcpyAsync(v_, vt, bytes, cudaMemcpyDeviceToDevice, s_));
    MD_CHECK(cudaStreamSynchronize(s_));
    cudaFree(xt);
    cudaFree(vt);
    step_ = s0;
    rec_count_ = r0;
    rec_last_step_ = l0;
    rec_interval_ = rec;
    forces_valid_ = false;
    rep << "chosen: list skin " << best << " nm (" << best_ms << " ms/step)\n";
    return rep.str();
}

void MDDriver::get_state(double* pos, double* vel, double* forces, double* potential, double* kinetic,
                         double* results) {
    MD_CHECK(cudaSetDevice(dev_));
    if ((forces || potential || kinetic || results) && !forces_valid_) compute_forces(true);
    MD_CHECK(cudaStreamSynchronize(s_terms_));  // the group-0 forces and energies below
    if (pos) MD_CHECK(cudaMemcpy(pos, x_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToHost));
    if (vel) MD_CHECK(cudaMemcpy(vel, v_, sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToHost));
    if (forces) {
        std::vector<unsigned long long> fb(3 * (size_t)n_);
        MD_CHECK(cudaMemcpy(forces, eng_->forces_device(), sizeof(double) * 3 * (size_t)n_, cudaMemcpyDeviceToHost));
        MD_CHECK(cudaMemcpy(fb.data(), fb_, sizeof(unsigned long long) * fb.size(), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < fb.size(); k++) forces[k] += (double)(long long)fb[k] / kFixScale;
    }
    std::vector<double> res((size_t)R_ * NUM_RES);
    if (potential || results)
        MD_CHECK(cudaMemcpy(res.data(), eng_->results_device(), sizeof(double) * res.size(), cudaMemcpyDeviceToHost));
    if (results) std::memcpy(results, res.data(), sizeof(double) * res.size());
    if (potential) {
        std::vector<double> et(term_rep_.size());
        if (!et.empty())
            MD_CHECK(cudaMemcpy(et.data(), e_terms_, sizeof(double) * et.size(), cudaMemcpyDeviceToHost));
        for (int r = 0; r < R_; r++) potential[r] = res[(size_t)r * NUM_RES + RES_ENERGY];
        for (size_t t = 0; t < et.size(); t++) potential[term_rep_[t]] += et[t];
    }
    if (kinetic) {
        MdDev a = dev_args();
        // on-step velocities v + (dt/2) f/m with their components along the constraints removed
        k_md_shift<<<(n_ + 255) / 256, 256, 0, s_>>>(a, xn_);
        if (n_cons_ + n_settle_ > 0) k_md_vproject<<<(n_cons_ + n_settle_ + 127) / 128, 128, 0, s_>>>(a, xn_);
        k_md_kinetic<<<R_, 256, 0, s_>>>(a, xn_);
        MD_CHECK(cudaGetLastError());
        MD_CHECK(cudaMemcpyAsync(kinetic, ke_d_, sizeof(double) * R_, cudaMemcpyDeviceToHost, s_));
        MD_CHECK(cudaStreamSynchronize(s_));
    }
}

}  // namespace atm
