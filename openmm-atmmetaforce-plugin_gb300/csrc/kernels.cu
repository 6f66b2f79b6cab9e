// CUDA kernels of the ATM evaluation path (sm_103a).
//
// Data flow of one evaluation of R replicas:
//   prepare  : user positions (FP64) -> wrapped float4 slots, state-2 copies,
//              block bounding boxes; zero the force accumulators
//   find     : one warp per tile row -> compacted list of interacting 32x32 tiles
//   tiles    : persistent warps over the tile list: LJ + reaction field / Ewald
//              direct space, tile rotation by warp shuffles, fixed-point forces
//   exceptions: exception pairs and Ewald exclusion corrections in FP64
//   spread / convert / (cuFFT R2C) / conv / (cuFFT C2R) / gather : smooth PME
//   finalize : FP64 energies, soft-core + softplus merge (ATM scalars)
//   output   : hybrid forces F1 + s' (F2 - F1) in user order
//   matrix   : replicas x states reduced-energy matrix
//
// Reference semantics: inner evaluations of ATMMetaForceImpl.cpp:113,116; the
// displacement of CopyState, platforms/common/src/kernels/atmmetaforce.cc:19-52;
// the merge of ReferenceATMMetaForceKernels.cpp:56-113 (FP64, as the Reference
// platform, instead of the float `sp` of CommonATMMetaForceKernels.cpp:199).
#include <cmath>
#include <cstdio>

#include "kernels.cuh"

namespace atm {

#define FULL_MASK 0xffffffffu

__device__ __forceinline__ void fix_add(unsigned long long* p, float v) {
    // the sum of two's-complement integers is exact and order independent
    atomicAdd(p, fix_bits(v));
}

__device__ __forceinline__ void fix_add_d(unsigned long long* p, double v) {
    atomicAdd(p, (unsigned long long)__double2ll_rn(v * kFixScale));
}

__device__ __forceinline__ float wrapf(float x, float L, float iL) { return x - L * floorf(x * iL); }

// ---------------------------------------------------------------------------
// prepare: one warp per block
// ---------------------------------------------------------------------------
// Bounding box of a block (minimum image relative to its first atom); h.w
// receives the number of real (non-padding) atoms of the block.
__device__ __forceinline__ void warp_bbox(float x, float y, float z, const RepDev& R, float4* c, float4* h,
                                          int lane, int nreal) {
    float x0 = __shfl_sync(FULL_MASK, x, 0), y0 = __shfl_sync(FULL_MASK, y, 0), z0 = __shfl_sync(FULL_MASK, z, 0);
    float dx = x - x0, dy = y - y0, dz = z - z0;
    min_image3(dx, dy, dz, R);
    float lx = dx, ly = dy, lz = dz, hx = dx, hy = dy, hz = dz;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(FULL_MASK, lx, o));
        ly = fminf(ly, __shfl_xor_sync(FULL_MASK, ly, o));
        lz = fminf(lz, __shfl_xor_sync(FULL_MASK, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(FULL_MASK, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(FULL_MASK, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(FULL_MASK, hz, o));
    }
    if (lane == 0) {
        *c = make_float4(x0 + 0.5f * (lx + hx), y0 + 0.5f * (ly + hy), z0 + 0.5f * (lz + hz), 0.f);
        *h = make_float4(0.5f * (hx - lx), 0.5f * (hy - ly), 0.5f * (hz - lz), __int_as_float(nreal));
    }
}

__global__ void k_prepare(Args a) {
    int lane = threadIdx.x & 31;
    int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (b >= a.NB) return;
    int s = b * kTile + lane;
    int rep = a.block_rep[b];
    const RepDev& R = a.reps[rep];
    int o = a.orig[s];
    const int nreal = __popc(__ballot_sync(FULL_MASK, o >= 0));  // padding sits at the end of a block
    if (o < 0) o = a.orig[b * kTile];  // padding copies the block's first atom
    const double* p = (a.io[0] ? a.io[0] : a.pos_in) + 3 * (size_t)(R.in_off + o);
    double xd = p[0], yd = p[1], zd = p[2];
    float x = (float)xd, y = (float)yd, z = (float)zd;
    // a position whose reduced coordinates lie safely inside (0, 1) (by 1e-5, far
    // beyond the FP32 estimate's error) is in the unit cell already: the FP64 wrap
    // would subtract zero.  Others take the FP64 wrap (FP64 is 1/64 of the FP32
    // rate on this part).
    constexpr float kIn = 1e-5f;
    const float ux = x * R.ibox[0], uy = y * R.ibox[1], uz = z * R.ibox[2];
    if (!(ux >= kIn && ux <= 1.0f - kIn && uy >= kIn && uy <= 1.0f - kIn && uz >= kIn && uz <= 1.0f - kIn)) {
        wrap3d(xd, yd, zd, R);  // FP64 wrap into the unit cell
        x = (float)xd;
        y = (float)yd;
        z = (float)zd;
    }
    float q = a.qs[s];
    a.posq[s] = make_float4(x, y, z, q);
    if (a.skin_half2 > 0.f) {
        // displacement since the last list build (minimum image: wrapping is no motion)
        const float4 r = a.posq_ref[s];
        float dx = x - r.x, dy = y - r.y, dz = z - r.z;
        min_image3(dx, dy, dz, R);
        float d2 = dx * dx + dy * dy + dz * dz;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(FULL_MASK, d2, o));
        // non-negative floats order as their bit patterns
        if (lane == 0) atomicMax(&a.status->disp2, __float_as_uint(d2));
    }
    for (int k = 0; k < 6; k++) a.F[(size_t)k * a.NA + s] = 0ull;
    if (a.adjoint)
        for (int k = 0; k < 3; k++) a.D[(size_t)k * a.NA + s] = 0ull;
    warp_bbox(x, y, z, R, &a.bb_c[b], &a.bb_h[b], lane, nreal);
    if (R.tric && lane == 0) {  // (lane 0 wrote the box)
        const float4 h = a.bb_h[b];
        atomicMax(&a.rep_hmax[rep], __float_as_uint(sqrtf(h.x * h.x + h.y * h.y + h.z * h.z)));
    }
    if (a.full) {
        float4 d = a.displ[s];
        float x2 = x + d.x, y2 = y + d.y, z2 = z + d.z;
        wrap3(x2, y2, z2, R);
        a.posq2[s] = make_float4(x2, y2, z2, q);
        warp_bbox(x2, y2, z2, R, &a.bb_c2[b], &a.bb_h2[b], lane, nreal);
        if (R.tric && lane == 0) {
            const float4 h = a.bb_h2[b];
            atomicMax(&a.rep_hmax[rep], __float_as_uint(sqrtf(h.x * h.x + h.y * h.y + h.z * h.z)));
        }
    }
    if (b == 0 && lane == 0) a.status->next_tile = 0;
}

void launch_prepare(const Args& a, cudaStream_t s) {
    int threads = 256;
    int blocks = (a.NB * 32 + threads - 1) / threads;
    k_prepare<<<blocks, threads, 0, s>>>(a);
}

// Whether this evaluation builds the lists: when forced, with no skin, or when an
// atom has moved more than skin / 2 since the last build (then no pair within the
// cutoff now was beyond rc + skin then).  A build resets the finder's counters.
__global__ void k_decide(Args a) {
    if (threadIdx.x != 0) return;
    Status* st = a.status;
    const float d2 = __uint_as_float(st->disp2);
    const bool build = a.list_ctl[0] != 0 || !(a.skin_half2 > 0.f) || d2 > a.skin_half2;
    st->sticky |= st->overflow;
    if (build) {
        st->tile_count = 0;
        st->overflow = 0;
        st->max_row = 0;
    }
    st->next_row = 0;  // the fused kernel walks the rows at every evaluation
    st->rebuild = build ? 1 : 0;
    st->disp2 = 0u;
    a.list_counts[0]++;
    if (build) a.list_counts[1]++;
}

void launch_decide(const Args& a, cudaStream_t s) { k_decide<<<1, 32, 0, s>>>(a); }

// ---------------------------------------------------------------------------
// find: one warp per row; bounding-box test of block I against candidates J
// ---------------------------------------------------------------------------
// (the tile finder and the pair-tile kernel live in tiles.cu)

// ---------------------------------------------------------------------------
// exceptions: user-order positions; one CTA per 256 exceptions of a replica.
// Pairs whose two atoms move together have the same separation in both states:
// their terms are evaluated once, in FP32 (FP64 sums), and enter state 2 with the
// identical value, so they cancel exactly in u.  Pairs across displacement
// classes change with the displacement and stay in FP64.
// ---------------------------------------------------------------------------
// One exception pair at separation (dx, dy, dz): energy, force on j (f), and
// (gcorr) erf(alpha r)/r of its Ewald exclusion correction.
__device__ __forceinline__ double exc_term(const Args& a, const RepDev& R, const ExcParam& p, double dx, double dy,
                                           double dz, double* f, double* gcorr) {
    *gcorr = 0.0;
    double r2 = dx * dx + dy * dy + dz * dz;
    double e = 0.0, fr = 0.0;
    if (p.x != 0.0 || p.z != 0.0) {
        // nonzero exception: Coulomb chargeProd/r + LJ, no cutoff, no periodic image
        double inv_r2 = 1.0 / r2, inv_r = sqrt(inv_r2);
        e += p.x * inv_r;
        fr += p.x * inv_r * inv_r2;
        if (p.z != 0.0) {
            double s2 = p.y * p.y * inv_r2;
            double s6 = s2 * s2 * s2;
            e += 4.0 * p.z * (s6 * s6 - s6);
            fr += 4.0 * p.z * (12.0 * s6 * s6 - 6.0 * s6) * inv_r2;
        }
    }
    f[0] = fr * dx;
    f[1] = fr * dy;
    f[2] = fr * dz;
    if (a.method == 4) {
        // Ewald exclusion correction at the minimum-image separation
        double mx = dx, my = dy, mz = dz;
        min_image3d(mx, my, mz, R);
        double m2 = mx * mx + my * my + mz * mz;
        if (m2 > 0.0) {
            double r = sqrt(m2);
            double ar = a.alphad * r;
            double ef = erf(ar);
            e -= p.w * ef / r;
            *gcorr = ef / r;
            double fm = p.w * (1.1283791670955126 * a.alphad * exp(-ar * ar) - ef / r) / m2;
            f[0] += fm * mx;
            f[1] += fm * my;
            f[2] += fm * mz;
        } else {
            e -= p.w * 1.1283791670955126 * a.alphad;
            *gcorr = 1.1283791670955126 * a.alphad;
        }
    }
    return e;
}

// FP32 form of exc_term for pairs within one displacement class.
__device__ __forceinline__ float exc_term_f(const Args& a, const RepDev& R, const ExcParam& p, float dx, float dy,
                                            float dz, float* f) {
    float r2 = dx * dx + dy * dy + dz * dz;
    float e = 0.0f, fr = 0.0f;
    float px = (float)p.x, pz = (float)p.z;
    if (px != 0.0f || pz != 0.0f) {
        float inv_r2 = 1.0f / r2, inv_r = sqrtf(inv_r2);
        e += px * inv_r;
        fr += px * inv_r * inv_r2;
        if (pz != 0.0f) {
            float py = (float)p.y;
            float s2 = py * py * inv_r2;
            float s6 = s2 * s2 * s2;
            e += 4.0f * pz * (s6 * s6 - s6);
            fr += 4.0f * pz * (12.0f * s6 * s6 - 6.0f * s6) * inv_r2;
        }
    }
    f[0] = fr * dx;
    f[1] = fr * dy;
    f[2] = fr * dz;
    if (a.method == 4) {
        float pw = (float)p.w;
        float mx = dx, my = dy, mz = dz;
        min_image3(mx, my, mz, R);
        float m2 = mx * mx + my * my + mz * mz;
        if (m2 > 0.0f) {
            float r = sqrtf(m2);
            float ar = a.alpha * r;
            float ef = erff(ar);
            e -= pw * ef / r;
            float fm = pw * (1.1283791670955126f * a.alpha * expf(-ar * ar) - ef / r) / m2;
            f[0] += fm * mx;
            f[1] += fm * my;
            f[2] += fm * mz;
        } else {
            e -= pw * 1.1283791670955126f * a.alpha;
        }
    }
    return e;
}

__global__ void __launch_bounds__(256) k_exceptions(Args a) {
    __shared__ double red[3][8];
    int c = blockIdx.x;
    int e = a.exc_cta_first[c] + threadIdx.x;
    float E1f = 0.0f;  // same-class pairs (FP32 terms, summed in FP32 within a warp)
    double E1 = 0.0, E2 = 0.0, DE = 0.0;
    if (e < a.exc_cta_first[c + 1]) {
        int4 ij = a.exc_ij[e];
        ExcParam p = a.exc_p[e];
        const RepDev& R = a.reps[ij.z];
        const double* pos = a.io[0] ? a.io[0] : a.pos_in;
        const double* xi = pos + 3 * (size_t)ij.x;
        const double* xj = pos + 3 * (size_t)ij.y;
        int si = a.slot_of[ij.x], sj = a.slot_of[ij.y];
        if (!ij.w) {
            float g[3];
            E1f = exc_term_f(a, R, p, (float)(xj[0] - xi[0]), (float)(xj[1] - xi[1]), (float)(xj[2] - xi[2]), g);
            for (int k = 0; k < 3; k++) {
                fix_add(a.F + (size_t)k * a.NA + si, -g[k]);
                fix_add(a.F + (size_t)k * a.NA + sj, g[k]);
            }
            if (a.full) {
                for (int k = 0; k < 3; k++) {
                    fix_add(a.F + (size_t)(3 + k) * a.NA + si, -g[k]);
                    fix_add(a.F + (size_t)(3 + k) * a.NA + sj, g[k]);
                }
            }
        } else {
            const double* di = a.displ_in + 3 * (size_t)ij.x;
            const double* dj = a.displ_in + 3 * (size_t)ij.y;
            double f1[3], f2[3], g1, g2;
            E1 = exc_term(a, R, p, xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2], f1, &g1);
            for (int k = 0; k < 3; k++) {
                fix_add_d(a.F + (size_t)k * a.NA + si, -f1[k]);
                fix_add_d(a.F + (size_t)k * a.NA + sj, f1[k]);
            }
            E2 = exc_term(a, R, p, (xj[0] + dj[0]) - (xi[0] + di[0]), (xj[1] + dj[1]) - (xi[1] + di[1]),
                          (xj[2] + dj[2]) - (xi[2] + di[2]), f2, &g2);
            if (!a.full) {
                DE = E2 - E1;
                E2 = 0.0;
                for (int k = 0; k < 3; k++) f2[k] -= f1[k];
                if (a.adjoint) {
                    // the exclusion correction -q_i q_j erf(alpha r)/r in scaled charges
                    fix_add_d(a.D + si, -(double)a.qs[sj] * (g2 - g1));
                    fix_add_d(a.D + sj, -(double)a.qs[si] * (g2 - g1));
                }
            }
            for (int k = 0; k < 3; k++) {
                fix_add_d(a.F + (size_t)(3 + k) * a.NA + si, -f2[k]);
                fix_add_d(a.F + (size_t)(3 + k) * a.NA + sj, f2[k]);
            }
        }
    }
    // fixed-order sums: FP32 same-class terms within the warp, FP64 from there on;
    // in two-state mode the same-class terms enter both states identically
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) E1f += __shfl_xor_sync(FULL_MASK, E1f, o);
    const bool any_cross = __any_sync(FULL_MASK, E1 != 0.0 || E2 != 0.0 || DE != 0.0);
    if (any_cross) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            E1 += __shfl_xor_sync(FULL_MASK, E1, o);
            E2 += __shfl_xor_sync(FULL_MASK, E2, o);
            DE += __shfl_xor_sync(FULL_MASK, DE, o);
        }
    }
    if (lane == 0) {
        red[0][w] = E1 + (double)E1f;
        red[1][w] = E2 + (a.full ? (double)E1f : 0.0);
        red[2][w] = DE;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int q = 0; q < 8; q++) t += red[threadIdx.x][q];
        a.e_part_exc[3 * c + threadIdx.x] = t;
    }
}

void launch_exceptions(const Args& a, cudaStream_t s) {
    if (a.exc_ctas > 0) k_exceptions<<<a.exc_ctas, 256, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// PME
// ---------------------------------------------------------------------------

// Order-5 cardinal B-spline weights w[k] = M5(t+k) and derivatives, by the
// recursion M_m(x) = (x M_{m-1}(x) + (m-x) M_{m-1}(x-1)) / (m-1).
__device__ __forceinline__ void bspline5(float t, float* w, float* dw) {
    float a0 = t, a1 = 1.0f - t;
    float b0 = 0.5f * t * a0, b1 = 0.5f * ((t + 1.0f) * a1 + (2.0f - t) * a0), b2 = 0.5f * (1.0f - t) * a1;
    const float third = 1.0f / 3.0f;
    float c0 = third * t * b0;
    float c1 = third * ((t + 1.0f) * b1 + (3.0f - t) * b0);
    float c2 = third * ((t + 2.0f) * b2 + (2.0f - t) * b1);
    float c3 = third * (1.0f - t) * b2;
    if (dw) {
        dw[0] = c0;
        dw[1] = c1 - c0;
        dw[2] = c2 - c1;
        dw[3] = c3 - c2;
        dw[4] = -c3;
    }
    w[0] = 0.25f * t * c0;
    w[1] = 0.25f * ((t + 1.0f) * c1 + (4.0f - t) * c0);
    w[2] = 0.25f * ((t + 2.0f) * c2 + (3.0f - t) * c1);
    w[3] = 0.25f * ((t + 3.0f) * c3 + (2.0f - t) * c2);
    w[4] = 0.25f * (1.0f - t) * c3;
}

struct Stencil {
    int base[3];
    float w[3][5];
    float dw[3][5];
};

__device__ __forceinline__ void make_stencil(float x, float y, float z, const RepDev& R, Stencil& S, bool deriv) {
    float fr[3];
    frac3(x, y, z, R, fr);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        float f = fr[d];
        f -= floorf(f);
        float u = f * (float)R.K[d];
        int b = (int)floorf(u);
        float t = u - (float)b;
        if (b >= R.K[d]) b -= R.K[d];
        if (b < 0) b += R.K[d];
        S.base[d] = b;
        bspline5(t, S.w[d], deriv ? S.dw[d] : nullptr);
    }
}

// Charge spreading by bricks.  One CTA holds one brick (the tuned edge, 12 to 20
// points) of one of a replica's two charge grids and adds stencils into an int32
// fixed-point accumulator in shared memory (2^25 units per e: integer sums are
// exact and order independent, so the grid is bit-reproducible), one atom per
// warp at a time with the lanes on its 5x5 (y, z) offsets; candidate atoms come
// from block bounding boxes in grid units (one point of margin for rounding).
//   By owner (spread_owner, the default where the grids allow it): the brick
//   takes the atoms whose stencil base it holds, each atom is spread once, into an
//   accumulator padded by the 4-point stencil reach below the brick, and the whole
//   accumulator is added to the grid (zeroed before) by integer atomics, the reach
//   landing in the neighbouring bricks' points.
//   By every touching brick: the brick takes every atom whose stencil reaches it,
//   padded by 4 points on each side, and writes only its own points, each once;
//   the padding belongs to the neighbouring bricks, which add the same atoms
//   themselves.  Grids smaller than a padded brick use the copy unpadded, with
//   per-point tests.
// Both sum the same integer contributions into each point.  Grid 0: state 1.
// Grid 1: the structure-factor update of the moving atoms, -q at x and +q at
// x + d, in both modes (state 2's grid is Q1 + dQ exactly: the non-moving atoms
// sit at the same grid points in both states and the integer sums are exact).
constexpr int kBrickThreads = 256;
constexpr int kBrickWarps = kBrickThreads / 32;
constexpr int kBrickPad = kOrder - 1;      // stencil reach below and above a brick

// Does the cyclic range of base indices of a box (fractional centre fc and half
// width fh along one box vector) meet the cyclic interval [o, o + len) of Z_K?
__device__ __forceinline__ bool cyc_meet(float fc, float fh, int K, int o, int len) {
    const int lo = (int)floorf((fc - fh) * (float)K) - 1;
    const int n = (int)floorf((fc + fh) * (float)K) + 1 - lo + 1;
    if (n >= K) return true;
    int A = lo % K;
    if (A < 0) A += K;
    int d1 = o - A;
    if (d1 < 0) d1 += K;
    int d2 = A - o;
    if (d2 < 0) d2 += K;
    return d1 < n || d2 < len;
}

// A block's bounding box (centre c, half extents h, nm) in fractional coordinates:
// centre p . r_d, half width sum_i h_i |r[i][d]| (r the reciprocal box).  Can an
// atom of the block have its stencil base in [o, o + e + reach) along every
// dimension (reach 4: its stencil touches the brick; 0: the brick owns it)?
__device__ __forceinline__ bool box_meets_brick(float4 c, float4 h, const RepDev& R, const int* o, const int* e,
                                                int reach) {
    float f[3];
    frac3(c.x, c.y, c.z, R, f);
    const float w0 = h.x * fabsf(R.recip[0]) + h.y * fabsf(R.recip[1]) + h.z * fabsf(R.recip[3]);
    const float w1 = h.y * fabsf(R.recip[2]) + h.z * fabsf(R.recip[4]);
    const float w2 = h.z * fabsf(R.recip[5]);
    return cyc_meet(f[0], w0, R.K[0], o[0], e[0] + reach) && cyc_meet(f[1], w1, R.K[1], o[1], e[1] + reach) &&
           cyc_meet(f[2], w2, R.K[2], o[2], e[2] + reach);
}

constexpr int kSpreadChunk = kBrickThreads;  // blocks examined per pass (one per thread)
constexpr int kSpreadCandCap = 2048;         // candidate entries listed before they are added
constexpr int kStencilWords = 16;            // q*wx[5], wy[5], wz[5], packed bases

// Dynamic shared memory of a spreading CTA: the brick accumulator (accum_bytes)
// plus each warp's 32 staged stencils.
int spread_smem_bytes(int accum_bytes) { return accum_bytes + kBrickWarps * 32 * kStencilWords * (int)sizeof(float); }

// Local index of grid point base - k in a brick [o, o + e), or -1.
__device__ __forceinline__ int brick_local(int base, int k, int o, int e, int K) {
    int v = base - k - o;
    v += v < 0 ? K : 0;
    v += v < 0 ? K : 0;
    return v < e ? v : -1;
}

// Adds the stencils of the atoms of candidate blocks s_cand[0 .. nc) to the brick
// accumulator: warp w takes candidates w, w + 8, ...; lanes = the block's atoms.
// An atom is added when its stencil base lies in [o, o + e + reach) (reach 4: its
// stencil touches the brick; 0: the brick owns it).
__device__ __forceinline__ void spread_candidates(const Args& a, const RepDev& R, const int* s_cand, int nc, int warp,
                                                  int lane, const int* o, const int* e, int pad, bool padded, int P1,
                                                  int P2, int* acc, float* st, int b0, int c0, int reach) {
    for (int ci = warp; ci < nc; ci += kBrickWarps) {
        const int ent = s_cand[ci];
        const int Jc = ent >> 2, code = ent & 3;
        const int s = Jc * kTile + lane;
        const int nreal = __float_as_int(a.bb_h[Jc].w);
        float4 p = code == 2 ? a.posq2[s] : a.posq[s];
        if (code == 1) p.w = -p.w;
        if (code == 3) {
            const float4 dd = a.displ[s];
            p.x += dd.x;
            p.y += dd.y;
            p.z += dd.z;
            wrap3(p.x, p.y, p.z, R);
        }
        bool ok = lane < nreal && p.w != 0.0f;
        int lb[3];
        if (ok) {
            float cc[3];
            frac3(p.x, p.y, p.z, R, cc);
#pragma unroll
            for (int d = 0; d < 3; d++) {
                float f = cc[d];
                f -= floorf(f);
                int bs = (int)floorf(f * (float)R.K[d]);
                if (bs >= R.K[d]) bs -= R.K[d];
                int v = bs - o[d];
                v += v < 0 ? R.K[d] : 0;
                ok = ok && v < e[d] + reach;
                lb[d] = v + pad;  // local index of the stencil's top point (padded copy)
            }
        }
        if (ok) {
            Stencil S;
            make_stencil(p.x, p.y, p.z, R, S, false);
            float* w = st + lane * kStencilWords;
            const float qs = p.w * kGridScale;
#pragma unroll
            for (int k = 0; k < kOrder; k++) {
                w[k] = qs * S.w[0][k];
                w[kOrder + k] = S.w[1][k];
                w[2 * kOrder + k] = S.w[2][k];
            }
            w[15] = __int_as_float(padded ? ((lb[0] << 20) | (lb[1] << 10) | lb[2])
                                          : ((S.base[0] << 20) | (S.base[1] << 10) | S.base[2]));
        }
        unsigned bal = __ballot_sync(FULL_MASK, ok);
        __syncwarp();
        // 3. the listed atoms one by one, lanes over the 5 x 5 (y, z) offsets
        while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            const float* w = st + src * kStencilWords;
            if (lane < kOrder * kOrder) {
                const int bases = __float_as_int(w[15]);
                const float wyz = w[kOrder + b0] * w[2 * kOrder + c0];
                if (padded) {
                    const int ly = ((bases >> 10) & 1023) - b0, lz = (bases & 1023) - c0;
                    const int row = ly * P2 + lz, lx0 = bases >> 20;
#pragma unroll
                    for (int a0 = 0; a0 < kOrder; a0++)
                        atomicAdd(&acc[(lx0 - a0) * P1 * P2 + row], __float2int_rn(w[a0] * wyz));
                } else {
                    const int ly = brick_local((bases >> 10) & 1023, b0, o[1], e[1], R.K[1]);
                    const int lz = brick_local(bases & 1023, c0, o[2], e[2], R.K[2]);
                    if (ly >= 0 && lz >= 0) {
                        const int bx = bases >> 20;
#pragma unroll
                        for (int a0 = 0; a0 < kOrder; a0++) {
                            const int lx = brick_local(bx, a0, o[0], e[0], R.K[0]);
                            if (lx >= 0) atomicAdd(&acc[(lx * P1 + ly) * P2 + lz], __float2int_rn(w[a0] * wyz));
                        }
                    }
                }
            }
            __syncwarp();
        }
    }
}

__global__ void __launch_bounds__(kBrickThreads) k_spread(Args a) {
    extern __shared__ int s_dyn[];
    __shared__ int s_cand[kSpreadCandCap];
    __shared__ int s_wcount[kBrickWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int c = blockIdx.x;
    const RepDev& R = a.reps[a.brick_cta_rep[c]];
    const int nb = R.nbrick[0] * R.nbrick[1] * R.nbrick[2];
    const int local = c - R.brick_cta_b;
    const int g = local / nb, b = local % nb;
    const int bi[3] = {b / (R.nbrick[1] * R.nbrick[2]), (b / R.nbrick[2]) % R.nbrick[1], b % R.nbrick[2]};
    int o[3], e[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        o[d] = bi[d] * R.bsz[d];
        e[d] = min(R.bsz[d], R.K[d] - o[d]);
    }
    const int npts = e[0] * e[1] * e[2];
    const size_t G3 = (size_t)R.K[0] * R.K[1] * R.K[2];
    float* G = a.qreal + R.real_off + (size_t)g * G3;
    // owner mode: the brick spreads the atoms whose stencil base it holds into an
    // accumulator padded by the stencil reach below it, and adds all of it to the
    // int32 grid (zeroed before the launch); the grid must exceed a padded brick
    const bool owner = a.spread_owner != 0;
    const int reach = owner ? 0 : kOrder - 1;
    // grid 1, the structure-factor update, has only the moving blocks (the last
    // blocks of the replica); a brick none of them reaches is written as zeros
    const bool upd = g == 1;
    const int jbegin = upd ? R.mov_block_begin : R.block_begin;
    if (upd) {
        bool any = false;
        for (int J = jbegin + tid; J < R.block_end; J += kBrickThreads) {
            const float4 c1 = a.bb_c[J], h1 = a.bb_h[J], dd = a.block_d[J];
            const float4 c2 = make_float4(c1.x + dd.x, c1.y + dd.y, c1.z + dd.z, 0.f);
            any = any || box_meets_brick(c1, h1, R, o, e, reach) || box_meets_brick(c2, h1, R, o, e, reach);
        }
        if (!__syncthreads_or(any)) {
            if (!owner)
                for (int k = tid; k < npts; k += kBrickThreads) {
                    const int lx = k / (e[1] * e[2]), ly = (k / e[2]) % e[1], lz = k % e[2];
                    G[((size_t)(o[0] + lx) * R.K[1] + (o[1] + ly)) * R.K[2] + o[2] + lz] = 0.0f;
                }
            return;
        }
    }
    // padded copy when the grid is larger than a padded brick in every dimension
    // (owner mode: padded below only, and always)
    const bool padded = owner || (R.K[0] >= e[0] + 2 * kBrickPad && R.K[1] >= e[1] + 2 * kBrickPad &&
                                  R.K[2] >= e[2] + 2 * kBrickPad);
    const int pad = padded ? kBrickPad : 0;
    const int span = owner ? pad : 2 * pad;
    const int P0 = e[0] + span, P1 = e[1] + span, Q2 = e[2] + span, P2 = spread_row_stride(Q2);
    int* acc = s_dyn;
    float* st = (float*)(s_dyn + a.brick_smem / 4) + warp * 32 * kStencilWords;  // this warp's staged stencils
    for (int k = tid; k < P0 * P1 * P2; k += kBrickThreads) acc[k] = 0;
    __syncthreads();
    const int b0 = lane / kOrder, c0 = lane % kOrder;
    int ncand = 0;  // candidates listed and not yet added (the same in every thread)
    for (int base = jbegin; base < R.block_end; base += kSpreadChunk) {
        // 1. blocks whose bounding box reaches the brick, in block order
        const int J = base + tid;
        int ent0 = -1, ent1 = -1;
        if (J < R.block_end) {
            if (g == 0) {
                if (box_meets_brick(a.bb_c[J], a.bb_h[J], R, o, e, reach)) ent0 = J << 2;
            } else if (a.block_cls[J] != 0) {
                const float4 c1 = a.bb_c[J], h1 = a.bb_h[J], dd = a.block_d[J];
                const float4 c2 = make_float4(c1.x + dd.x, c1.y + dd.y, c1.z + dd.z, 0.f);
                if (box_meets_brick(c1, h1, R, o, e, reach)) ent0 = (J << 2) | 1;
                if (box_meets_brick(c2, h1, R, o, e, reach)) ent1 = (J << 2) | 3;
            }
        }
        const unsigned m0 = __ballot_sync(FULL_MASK, ent0 >= 0), m1 = __ballot_sync(FULL_MASK, ent1 >= 0);
        if (lane == 0) s_wcount[warp] = __popc(m0) + __popc(m1);
        __syncthreads();
        int off = 0, nc = 0;
#pragma unroll
        for (int q = 0; q < kBrickWarps; q++) {
            const int cq = s_wcount[q];
            off += q < warp ? cq : 0;
            nc += cq;
        }
        if (ncand + nc > kSpreadCandCap) {  // list full: add what is listed first
            spread_candidates(a, R, s_cand, ncand, warp, lane, o, e, pad, padded, P1, P2, acc, st, b0, c0, reach);
            __syncthreads();
            ncand = 0;
        }
        {
            const unsigned lt = (1u << lane) - 1u;
            int pos = ncand + off + __popc(m0 & lt) + __popc(m1 & lt);
            if (ent0 >= 0) s_cand[pos++] = ent0;
            if (ent1 >= 0) s_cand[pos] = ent1;
        }
        ncand += nc;
        __syncthreads();
    }
    // 2. all listed candidates at once (one barrier for the whole brick)
    spread_candidates(a, R, s_cand, ncand, warp, lane, o, e, pad, padded, P1, P2, acc, st, b0, c0, reach);
    __syncthreads();
    if (owner) {
        // 4. the whole accumulator, the brick's points and the reach below it, added
        // to the int32 grid (integer sums: exact and order independent)
        int* Gi = reinterpret_cast<int*>(G);
        const int plane = P1 * Q2;
        for (int k = tid; k < P0 * plane; k += kBrickThreads) {
            const int lx = k / plane, r = k - lx * plane, ly = r / Q2, lz = r - ly * Q2;
            const int v = acc[(lx * P1 + ly) * P2 + lz];
            if (v == 0) continue;
            int gx = o[0] - pad + lx, gy = o[1] - pad + ly, gz = o[2] - pad + lz;
            gx += gx < 0 ? R.K[0] : 0;
            gy += gy < 0 ? R.K[1] : 0;
            gz += gz < 0 ? R.K[2] : 0;
            atomicAdd(Gi + ((size_t)gx * R.K[1] + gy) * R.K[2] + gz, v);
        }
        return;
    }
    // 4. the brick's own points, each written once
    for (int k = tid; k < npts; k += kBrickThreads) {
        const int lx = k / (e[1] * e[2]), ly = (k / e[2]) % e[1], lz = k % e[2];
        const int v = acc[((lx + pad) * P1 + ly + pad) * P2 + lz + pad];
        G[((size_t)(o[0] + lx) * R.K[1] + (o[1] + ly)) * R.K[2] + o[2] + lz] = (float)v * (1.0f / kGridScale);
    }
}

// Spreading per atom, for systems too small to fill the GPU with bricks: a warp
// takes one block of 32 atoms (grid 0: every block at x; grid 1: every moving
// block at x with -q and at x + d with +q), each lane computes its atom's stencil,
// then the atoms one by one with the lanes on the 5 x 5 (y, z) offsets add their
// 125 points to the int32 grid by atomics.  The integer contribution of an atom to
// a point is computed exactly as the bricks compute it, so the grids are the same
// bits.
constexpr int kSpreadAtomWarps = 8;

__global__ void __launch_bounds__(kSpreadAtomWarps * 32) k_spread_atoms(Args a) {
    __shared__ float s_st[kSpreadAtomWarps][32 * kStencilWords];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int item = blockIdx.x * kSpreadAtomWarps + w;
    if (item >= a.NB + 2 * a.n_mov_blocks) return;
    int blk, code;  // 0: grid 0 at x; 1: grid 1, -q at x; 3: grid 1, +q at x + d
    if (item < a.NB) {
        blk = item;
        code = 0;
    } else {
        const int m = item - a.NB;
        blk = a.mov_blocks[m >> 1];
        code = (m & 1) ? 3 : 1;
    }
    const RepDev& R = a.reps[a.block_rep[blk]];
    const int s = blk * kTile + lane;
    const int nreal = __float_as_int(a.bb_h[blk].w);
    float4 p = a.posq[s];
    if (code == 1) p.w = -p.w;
    if (code == 3) {
        const float4 dd = a.displ[s];
        p.x += dd.x;
        p.y += dd.y;
        p.z += dd.z;
        wrap3(p.x, p.y, p.z, R);
    }
    const bool ok = lane < nreal && p.w != 0.0f;
    float* st = s_st[w];
    if (ok) {
        Stencil S;
        make_stencil(p.x, p.y, p.z, R, S, false);
        float* wv = st + lane * kStencilWords;
        const float qs = p.w * kGridScale;
#pragma unroll
        for (int k = 0; k < kOrder; k++) {
            wv[k] = qs * S.w[0][k];
            wv[kOrder + k] = S.w[1][k];
            wv[2 * kOrder + k] = S.w[2][k];
        }
        wv[15] = __int_as_float((S.base[0] << 20) | (S.base[1] << 10) | S.base[2]);
    }
    unsigned bal = __ballot_sync(FULL_MASK, ok);
    __syncwarp();
    const int K0 = R.K[0], K1 = R.K[1], K2 = R.K[2];
    int* G = reinterpret_cast<int*>(a.qreal + R.real_off + (code ? (size_t)K0 * K1 * K2 : 0));
    const int b0 = lane / kOrder, c0 = lane % kOrder;
    while (bal) {
        const int src = __ffs(bal) - 1;
        bal &= bal - 1;
        const float* wv = st + src * kStencilWords;
        if (lane < kOrder * kOrder) {
            const int bases = __float_as_int(wv[15]);
            int y = ((bases >> 10) & 1023) - b0, z = (bases & 1023) - c0;
            y += y < 0 ? K1 : 0;
            z += z < 0 ? K2 : 0;
            const float wyz = wv[kOrder + b0] * wv[2 * kOrder + c0];
            const int x0 = bases >> 20;
#pragma unroll
            for (int a0 = 0; a0 < kOrder; a0++) {
                int x = x0 - a0;
                x += x < 0 ? K0 : 0;
                atomicAdd(G + ((size_t)x * K1 + y) * K2 + z, __float2int_rn(wv[a0] * wyz));
            }
        }
    }
}

void launch_spread(const Args& a, cudaStream_t s) {
    if (a.spread_atoms) {
        cudaMemsetAsync(a.qreal, 0, sizeof(float) * (size_t)a.n_real_total, s);
        const int items = a.NB + 2 * a.n_mov_blocks;
        k_spread_atoms<<<(items + kSpreadAtomWarps - 1) / kSpreadAtomWarps, kSpreadAtomWarps * 32, 0, s>>>(a);
        return;
    }
    if (a.brick_ctas <= 0) return;
    // owner mode adds every brick into the grids: they start at zero
    if (a.spread_owner) cudaMemsetAsync(a.qreal, 0, sizeof(float) * (size_t)a.n_real_total, s);
    const int bytes = spread_smem_bytes(a.brick_smem);
    // opt in to more than 48 KB of dynamic shared memory (per device; this runs
    // when the evaluation graph is recorded, not at every evaluation)
    cudaFuncSetAttribute(k_spread, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    k_spread<<<a.brick_ctas, kBrickThreads, bytes, s>>>(a);
}

// reciprocal-space convolution on the half spectrum; energies per CTA
constexpr int kConvThreads = 256;
__global__ void __launch_bounds__(kConvThreads) k_conv(Args a) {
    __shared__ double red[2][kConvThreads];
    int c = blockIdx.x;
    const RepDev& R = a.reps[a.conv_cta_rep[c]];
    const int Kx = R.K[0], Ky = R.K[1], Kz = R.K[2];
    const int Kzh = Kz / 2 + 1;
    const long long nc = (long long)Kx * Ky * Kzh;
    long long first = a.conv_cta_first[2 * c];
    long long last = a.conv_cta_first[2 * c + 1];
    float2* A = a.qcplx + R.cplx_off;
    float2* B = A + nc;
    const float* mx = a.moduli + R.mod_off[0];
    const float* my = a.moduli + R.mod_off[1];
    const float* mz = a.moduli + R.mod_off[2];
    const float pi = 3.14159265358979f;
    const float vol = R.box[0] * R.box[1] * R.box[2];
    const float pref = 1.0f / (pi * vol);
    const float fac = pi * pi / (a.alpha * a.alpha);
    // the reciprocal energies (and with them u) accumulate in FP64; each point's
    // term is an FP32 product
    double ea = 0.0, eb = 0.0;
    for (long long k = first + threadIdx.x; k < last; k += kConvThreads) {
        int iz = (int)(k % Kzh);
        long long rem = k / Kzh;
        int iy = (int)(rem % Ky);
        int ix = (int)(rem / Ky);
        int mxi = ix <= Kx / 2 ? ix : ix - Kx;
        int myi = iy <= Ky / 2 ? iy : iy - Ky;
        // m = mx a* + my b* + mz c* (the reciprocal vectors are the columns of the reciprocal box)
        float kx = mxi * R.recip[0], ky = fmaf(myi, R.recip[2], mxi * R.recip[1]),
              kz = fmaf(iz, R.recip[5], fmaf(myi, R.recip[4], mxi * R.recip[3]));
        float m2 = kx * kx + ky * ky + kz * kz;
        float G = (k == 0) ? 0.0f : pref * expf(-fac * m2) / (m2 * mx[ix] * my[iy] * mz[iz]);
        float wgt = (iz == 0 || 2 * iz == Kz) ? 1.0f : 2.0f;
        float2 qa = A[k], qb = B[k];
        float na = qa.x * qa.x + qa.y * qa.y;
        ea += (double)(0.5f * wgt * G * na);
        eb += (double)(wgt * G * (qa.x * qb.x + qa.y * qb.y + 0.5f * (qb.x * qb.x + qb.y * qb.y)));
        A[k] = make_float2(G * qa.x, G * qa.y);
        // grid 1 holds dQ: its potential is G dQ (difference mode) or state 2's, G (Q1 + dQ)
        B[k] = a.full ? make_float2(G * (qa.x + qb.x), G * (qa.y + qb.y)) : make_float2(G * qb.x, G * qb.y);
    }
    red[0][threadIdx.x] = ea;
    red[1][threadIdx.x] = eb;
    __syncthreads();
    for (int o = kConvThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x < 2) a.e_part_conv[2 * c + threadIdx.x] = red[threadIdx.x][0];
}

void launch_conv(const Args& a, cudaStream_t s) {
    k_conv<<<a.conv_ctas, kConvThreads, 0, s>>>(a);
}

__device__ __forceinline__ void gather_one(const float* G, const RepDev& R, const Stencil& S, float& gx, float& gy,
                                           float& gz, float* pot = nullptr) {
    float ph = 0.f;
    const int Kx = R.K[0], Ky = R.K[1], Kz = R.K[2];
    int iz[5];
#pragma unroll
    for (int c = 0; c < 5; c++) {
        int v = S.base[2] - c;
        iz[c] = v < 0 ? v + Kz : v;
    }
    gx = gy = gz = 0.f;
#pragma unroll
    for (int a0 = 0; a0 < 5; a0++) {
        int ix = S.base[0] - a0;
        if (ix < 0) ix += Kx;
#pragma unroll
        for (int b0 = 0; b0 < 5; b0++) {
            int iy = S.base[1] - b0;
            if (iy < 0) iy += Ky;
            const float* rowp = G + ((size_t)ix * Ky + iy) * Kz;
            float sx = 0.f, sz = 0.f;
#pragma unroll
            for (int c0 = 0; c0 < 5; c0++) {
                float v = __ldg(rowp + iz[c0]);
                sx += S.w[2][c0] * v;
                sz += S.dw[2][c0] * v;
            }
            gx += S.dw[0][a0] * S.w[1][b0] * sx;
            gy += S.w[0][a0] * S.dw[1][b0] * sx;
            gz += S.w[0][a0] * S.w[1][b0] * sz;
            if (pot) ph += S.w[0][a0] * S.w[1][b0] * sx;
        }
    }
    if (pot) *pot = ph;
}

__device__ __forceinline__ float pick5(const float* w, int k) {
    return k == 0 ? w[0] : k == 1 ? w[1] : k == 2 ? w[2] : k == 3 ? w[3] : k == 4 ? w[4] : 0.0f;
}

// Gradient of one grid at one stencil (and with POT the potential) with 16-byte
// loads: the five z points base - 4 .. base of every (x, y) row lie in the
// aligned eight-float window that starts at az = (base - 4) & ~3, read as two
// float4; the z weights are re-indexed into that window once.  Returns false
// (nothing computed) when the window would wrap around the grid; the grid must
// start 16-byte aligned with Kz a multiple of 4.
template <bool POT>
__device__ __forceinline__ bool gather_vec(const float* G, const RepDev& R, const Stencil& S, float* g, float* pot) {
    const int Kx = R.K[0], Ky = R.K[1], Kz = R.K[2];
    const int z0 = S.base[2] - (kOrder - 1);
    const int az = z0 & ~3;
    if (z0 < 0 || az + 8 > Kz) return false;
    const int m = z0 - az;  // 0..3
    float Wz[8], dWz[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int c = m + kOrder - 1 - k;  // z weight index of window entry k (-1..7 outside)
        Wz[k] = pick5(S.w[2], c);
        dWz[k] = pick5(S.dw[2], c);
    }
    float ax = 0.f, ay = 0.f, az_ = 0.f, ph = 0.f;
#pragma unroll
    for (int i0 = 0; i0 < kOrder; i0++) {
        int ix = S.base[0] - i0;
        if (ix < 0) ix += Kx;
#pragma unroll
        for (int j0 = 0; j0 < kOrder; j0++) {
            int iy = S.base[1] - j0;
            if (iy < 0) iy += Ky;
            const size_t ro = ((size_t)ix * Ky + iy) * Kz + az;
            const float dxy = S.dw[0][i0] * S.w[1][j0], xdy = S.w[0][i0] * S.dw[1][j0], xy = S.w[0][i0] * S.w[1][j0];
            const float4 lo = __ldg((const float4*)(G + ro)), hi = __ldg((const float4*)(G + ro + 4));
            const float sx = Wz[0] * lo.x + Wz[1] * lo.y + Wz[2] * lo.z + Wz[3] * lo.w + Wz[4] * hi.x +
                             Wz[5] * hi.y + Wz[6] * hi.z + Wz[7] * hi.w;
            const float sz = dWz[0] * lo.x + dWz[1] * lo.y + dWz[2] * lo.z + dWz[3] * lo.w + dWz[4] * hi.x +
                             dWz[5] * hi.y + dWz[6] * hi.z + dWz[7] * hi.w;
            ax += dxy * sx;
            ay += xdy * sx;
            az_ += xy * sz;
            if (POT) ph += xy * sx;
        }
    }
    g[0] = ax;
    g[1] = ay;
    g[2] = az_;
    if (POT) *pot = ph;
    return true;
}

// -q grad phi from the gradient g_d along the grid coordinates s_d = K_d (p . r_d):
// F_j = -q sum_d g_d K_d r[j][d] (r the reciprocal box, lower triangular).
__device__ __forceinline__ void add_grad_force(unsigned long long* F, int NA, int s, float q, float gx, float gy,
                                               float gz, const RepDev& R) {
    const float g0 = gx * (float)R.K[0], g1 = gy * (float)R.K[1], g2 = gz * (float)R.K[2];
    fix_add(F + s, -q * (g0 * R.recip[0]));
    fix_add(F + NA + s, -q * fmaf(g1, R.recip[2], g0 * R.recip[1]));
    fix_add(F + 2 * (size_t)NA + s, -q * fmaf(g2, R.recip[5], fmaf(g1, R.recip[4], g0 * R.recip[3])));
}

// Reciprocal-space forces of every atom that does not move (difference mode)
// or of every atom at both states (two-state mode).  Two threads per atom, one
// per grid (the two halves of a CTA: 64 atoms, grid 0 then grid 1), so that each
// thread holds one grid's sums and more warps hide the grid reads' latency.
constexpr int kGatherAtoms = 64;

// Gradient of one grid at a stencil (and with pot != nullptr its potential):
// the aligned float4 windows where they fit, single points otherwise.
__device__ __forceinline__ void gather_grid(const float* G, const RepDev& R, const Stencil& S, float* g, float* pot) {
    const bool vec = ((R.real_off | (long long)R.K[2]) & 3) == 0;
    if (pot) {
        if (!(vec && gather_vec<true>(G, R, S, g, pot))) gather_one(G, R, S, g[0], g[1], g[2], pot);
    } else {
        if (!(vec && gather_vec<false>(G, R, S, g, nullptr))) gather_one(G, R, S, g[0], g[1], g[2]);
    }
}

// The moving atoms of the difference mode, one CTA per moving block, warps 0-2
// on the three gathers of F1 at x in phi1 and F2 - F1 = F(x + d in phi1 + dphi)
// - F(x in phi1):  warp 0: phi1 at x (F1 += g, F2 -= g), warp 1: phi1 at x + d,
// warp 2: dphi at x + d (F2 += each).  Fixed-point sums: the order is immaterial.
__device__ __noinline__ void gather_moving(const Args& a, int blk) {
    const int w = threadIdx.x >> 5;
    if (w > 2) return;
    const int b = a.mov_blocks[blk];
    const int s = b * kTile + (threadIdx.x & 31);
    const RepDev& R = a.reps[a.block_rep[b]];
    const float4 p = a.posq[s];
    if (p.w == 0.0f) return;
    const size_t G3 = (size_t)R.K[0] * R.K[1] * R.K[2];
    const float* G = a.qreal + R.real_off + (w == 2 ? G3 : 0);
    Stencil S;
    if (w == 0) {
        make_stencil(p.x, p.y, p.z, R, S, true);
    } else {
        const float4 d = a.displ[s];
        float x2 = p.x + d.x, y2 = p.y + d.y, z2 = p.z + d.z;
        wrap3(x2, y2, z2, R);
        make_stencil(x2, y2, z2, R, S, true);
    }
    float g[3], pot = 0.f;
    gather_grid(G, R, S, g, a.adjoint ? &pot : nullptr);
    unsigned long long* F2 = a.F + 3 * (size_t)a.NA;
    if (w == 0) {
        add_grad_force(a.F, a.NA, s, p.w, g[0], g[1], g[2], R);
        add_grad_force(F2, a.NA, s, p.w, -g[0], -g[1], -g[2], R);
        if (a.adjoint) fix_add(a.D + s, -pot);  // potential at x + d in state 2 minus at x in state 1
    } else {
        add_grad_force(F2, a.NA, s, p.w, g[0], g[1], g[2], R);
        if (a.adjoint) fix_add(a.D + s, pot);
    }
}

__global__ void __launch_bounds__(2 * kGatherAtoms, 6) k_gather(Args a) {
    const int nmain = (a.NA + kGatherAtoms - 1) / kGatherAtoms;
    if ((int)blockIdx.x >= nmain) {
        gather_moving(a, blockIdx.x - nmain);
        return;
    }
    const int half = threadIdx.x / kGatherAtoms;  // warp-uniform
    const int s = blockIdx.x * kGatherAtoms + (threadIdx.x - half * kGatherAtoms);
    if (s >= a.NA) return;
    const int b = s >> 5;
    if (!a.full && a.block_cls[b] != 0) return;  // moving atoms: the CTAs after the first nmain
    const RepDev& R = a.reps[a.block_rep[b]];
    const float q = a.posq[s].w;
    if (q == 0.0f) return;
    const size_t G3 = (size_t)R.K[0] * R.K[1] * R.K[2];
    const float* G = a.qreal + R.real_off + (half ? G3 : 0);
    unsigned long long* F = a.F + (half ? 3 * (size_t)a.NA : 0);
    // two-state mode: grid 1 is state 2 at x + d; difference mode: the potential
    // of the moved charges at x (F2 - F1 and, for the adjoint, d(E2 - E1)_rec/dq)
    const float4 p = (a.full && half) ? a.posq2[s] : a.posq[s];
    Stencil S;
    make_stencil(p.x, p.y, p.z, R, S, true);
    float g[3], pot = 0.f;
    const bool with_pot = !a.full && half && a.adjoint;
    gather_grid(G, R, S, g, with_pot ? &pot : nullptr);
    if (with_pot) fix_add(a.D + s, pot);
    add_grad_force(F, a.NA, s, q, g[0], g[1], g[2], R);
}

void launch_gather(const Args& a, cudaStream_t s) {
    const int nmain = (a.NA + kGatherAtoms - 1) / kGatherAtoms;
    const int nmov = a.full ? 0 : a.n_mov_blocks;
    k_gather<<<nmain + nmov, 2 * kGatherAtoms, 0, s>>>(a);
}

// ---------------------------------------------------------------------------
// finalize: one CTA per replica, FP64
// ---------------------------------------------------------------------------

// SoftCoreF of ReferenceATMMetaForceKernels.cpp:26-37
__device__ double softcore(double u, double umax, double acore, double ub, double& fp) {
    if (u <= ub) {
        fp = 1.0;
        return u;
    }
    // (one thread per replica runs this FP64 chain, whose latency the evaluation
    // waits on: zeta^acore as exp(acore log zeta), 1/(1 + zeta^acore) taken once)
    double gu = (u - ub) / (acore * (umax - ub));
    double zeta = 1.0 + 2.0 * gu * (gu + 1.0);
    double zetap = exp(acore * log(zeta));
    double sf = 4.0 * (2.0 * gu + 1.0) / zeta;
    const double rz = 1.0 / (1.0 + zetap);
    fp = sf * zetap * rz * rz;
    return (umax - ub) * (zetap - 1.0) * rz + ub;
}

// The merge of ReferenceATMMetaForceKernels.cpp:82-98 plus the closed-form
// parameter derivatives of W.
__device__ void atm_merge(double E1, double E2, const double* p, double* out) {
    double l1 = p[0], l2 = p[1], alpha = p[2], u0 = p[3], w0 = p[4];
    double umax = p[5], ub = p[6], acore = p[7], dir = p[8];
    double u = dir > 0 ? E2 - E1 : E1 - E2;
    double e0 = dir > 0 ? E1 : E2;
    double fp;
    double usc = softcore(u, umax, acore, ub, fp);
    double x = exp(-alpha * (usc - u0));
    double ee = 1.0 + x;
    const double iee = 1.0 / ee, ia = alpha > 0 ? 1.0 / alpha : 0.0;
    double W = 0.0;
    double L = log(ee);
    if (alpha > 0) W = ((l2 - l1) * ia) * L;
    W += l2 * usc + w0;
    double bfp = (l2 - l1) * iee + l1;
    out[RES_ENERGY] = e0 + W;
    out[RES_PERT] = usc;
    out[RES_SP] = bfp * fp;
    out[RES_W] = W;
    out[RES_U] = u;
    out[RES_E0] = e0;
    out[RES_BFP] = bfp;
    out[RES_FP] = fp;
    out[RES_E1] = E1;
    out[RES_E2] = E2;
    if (alpha > 0) {
        out[RES_DL1] = -L * ia;
        out[RES_DL2] = L * ia + usc;
        out[RES_DALPHA] = -(l2 - l1) * (ia * ia) * L - (l2 - l1) * ia * (usc - u0) * x * iee;
        out[RES_DU0] = (l2 - l1) * x * iee;
    } else {
        out[RES_DL1] = 0.0;
        out[RES_DL2] = usc;
        out[RES_DALPHA] = 0.0;
        out[RES_DU0] = 0.0;
    }
    out[RES_DW0] = 1.0;
    // derivative of the W computed above (with alpha = 0 the log term is absent, so
    // dW/dusc = lambda2, not the bfp the force merge uses)
    out[RES_DWDU] = (alpha > 0 ? bfp : l2) * fp;
}

// Energies of a replica and the ATM merge, one kernel: CTA c of replica r sums
// the tile energies of the replica's rows c, c + C, ... (C = fin_ctas; rows of
// state 1, then rows of state 2 or of the difference tiles), warp per row, lanes
// over its slots, each lane in compensated FP32 (TwoSum: relative error of order
// 2^-48 of the summed magnitudes, on the FP32 pipe), the lanes' compensated pairs
// combined over a shuffle tree and converted to FP64 once per warp, then FP64
// across warps and CTAs, in a fixed order (no fixed-point range would do:
// the difference tiles of a displaced ligand that overlaps the solvent reach 1e10
// kJ/mol and more, which the soft-core exists to absorb), and writes its two
// partials; the last CTA of the replica to finish (a counter it resets for the
// next evaluation) adds the partials in order, the exceptions' and the
// reciprocal sum's partials, and runs the FP64 merge.
constexpr int kFinThreads = 256;

// Knuth's TwoSum: s + c carries the running sum exactly up to c's own rounding.
__device__ __forceinline__ void fin_two_sum(float& s, float& c, float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

// (h, l) += (hb, lb) for two compensated sums: TwoSum of the leading parts, the
// trailing parts added to its error, renormalised (Fast2Sum) so that the next
// combination's TwoSum sees the full leading part.
__device__ __forceinline__ void fin_pair_add(float& h, float& l, float hb, float lb) {
    const float s = h + hb;
    const float bp = s - h;
    const float t = ((h - (s - bp)) + (hb - bp)) + (l + lb);
    h = s + t;
    l = t - (h - s);
}

__global__ void __launch_bounds__(kFinThreads) k_finalize(Args a) {
    __shared__ double sh_r[2][kFinThreads / 32];
    __shared__ double sh[5][kFinThreads / 32];
    __shared__ int s_last;
    const int C = a.fin_ctas;
    const int r = blockIdx.x / C, c = blockIdx.x - r * C;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const RepDev& R = a.reps[r];
    const int n1 = R.row1_e - R.row1_b, n2 = R.row2_e - R.row2_b;
    float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;  // compensated sums of the two row kinds
    for (int k = c + C * w; k < n1 + n2; k += C * (kFinThreads / 32)) {
        const int row = k < n1 ? R.row1_b + k : R.row2_b + (k - n1);
        const int n = a.row_count[row];
        const float2* e = a.e_tile + (size_t)row * a.row_cap;
        const bool first = k < n1;
        for (int q = lane; q < n; q += 32) {
            const float2 v = e[q];
            if (first) {
                fin_two_sum(h1, l1, v.x);
                l1 += v.y;
            } else {
                fin_two_sum(h2, l2, v.x);
                l2 += v.y;
            }
        }
    }
    // across the warp as compensated pairs on the FP32 pipe, to FP64 once per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float hb1 = __shfl_xor_sync(FULL_MASK, h1, o), lb1 = __shfl_xor_sync(FULL_MASK, l1, o);
        const float hb2 = __shfl_xor_sync(FULL_MASK, h2, o), lb2 = __shfl_xor_sync(FULL_MASK, l2, o);
        fin_pair_add(h1, l1, hb1, lb1);
        fin_pair_add(h2, l2, hb2, lb2);
    }
    if (lane == 0) {
        sh_r[0][w] = (double)h1 + (double)l1;
        sh_r[1][w] = (double)h2 + (double)l2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t1 = 0.0, t2 = 0.0;
        for (int q = 0; q < kFinThreads / 32; q++) {
            t1 += sh_r[0][q];
            t2 += sh_r[1][q];
        }
        a.fin_part[2 * (size_t)blockIdx.x] = t1;
        a.fin_part[2 * (size_t)blockIdx.x + 1] = t2;
        __threadfence();
        s_last = atomicAdd(&a.fin_count[r], 1) == C - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // the replica's last CTA: partials of the rows (fixed order), the exceptions
    // (3) and the reciprocal sum (2)
    double v[5] = {0, 0, 0, 0, 0};
    for (int q = R.exc_cta_b + threadIdx.x; q < R.exc_cta_e; q += blockDim.x) {
        v[0] += a.e_part_exc[3 * q];
        v[1] += a.e_part_exc[3 * q + 1];
        v[2] += a.e_part_exc[3 * q + 2];
    }
    for (int q = R.conv_cta_b + threadIdx.x; q < R.conv_cta_e; q += blockDim.x) {
        v[3] += a.e_part_conv[2 * q];
        v[4] += a.e_part_conv[2 * q + 1];
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(FULL_MASK, v[k], o);
        if (lane == 0) sh[k][w] = v[k];
    }
    __syncthreads();
    if (w != 0) return;
    // warp 0: the CTAs' partials (lane q holds CTAs q, q + 32, ...) and the warps'
    // sums, each added over a fixed shuffle tree
    double dir1 = 0.0, dir2 = 0.0;
    {
        const volatile double* part = a.fin_part + 2 * (size_t)r * C;
        for (int q = lane; q < C; q += 32) {
            dir1 += part[2 * q];
            dir2 += part[2 * q + 1];
        }
    }
    double t[5];
#pragma unroll
    for (int k = 0; k < 5; k++) t[k] = lane < kFinThreads / 32 ? sh[k][lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dir1 += __shfl_xor_sync(FULL_MASK, dir1, o);
        dir2 += __shfl_xor_sync(FULL_MASK, dir2, o);
    }
#pragma unroll
    for (int o = (kFinThreads / 32) / 2; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 5; k++) t[k] += __shfl_xor_sync(FULL_MASK, t[k], o);
    if (lane == 0) {
        a.fin_count[r] = 0;  // ready for the next evaluation
        const double x1 = t[0], x2 = t[1], xd = t[2], c1 = t[3], c2 = t[4];
        double E1 = dir1 + x1 + c1 + R.e_self + R.e_disp;
        double E2;
        if (a.full) {
            // c2 = E_rec2 - E_rec1, summed directly from the structure-factor update
            E2 = dir2 + x2 + (c1 + c2) + R.e_self + R.e_disp;
        } else {
            E2 = E1 + (dir2 + xd + c2);
        }
        double* out = a.results + (size_t)r * NUM_RES;
        // a NonbondedForce outside the variable groups contributes nothing to U_var
        atm_merge(R.var_nb ? E1 : 0.0, R.var_nb ? E2 : 0.0, R.params, out);
        out[RES_E1] = E1;  // the NonbondedForce energy at x and at x + d
        out[RES_E2] = E2;
        out[RES_STATUS] = (double)a.status->overflow;
        if (a.io[2])
            for (int k = 0; k < NUM_RES; k++) a.io[2][(size_t)r * NUM_RES + k] = out[k];
    }
}

void launch_finalize(const Args& a, cudaStream_t s) {
    k_finalize<<<a.R * a.fin_ctas, kFinThreads, 0, s>>>(a);
}

// Hybrid forces in user order: thread g takes input atom g (its slot from
// slot_of), so that a warp's 32 atoms are 768 contiguous bytes of the output,
// written as 16-byte words through shared memory.  The output is f_out, or a
// page-locked host buffer the caller passed (io[1]), written over the host link
// without a separate copy.
constexpr int kOutThreads = 256;

__global__ void __launch_bounds__(kOutThreads) k_output(Args a) {
    __shared__ double s_f[kOutThreads / 32][96];
    const int g = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double* const fo = a.io[1] ? a.io[1] : a.f_out;
    double f[3] = {0.0, 0.0, 0.0};
    if (g < a.n_in) {
        const int s = a.slot_of[g];
        const int rep = a.block_rep[s >> 5];
        const RepDev& R = a.reps[rep];
        const double* res = a.results + (size_t)rep * NUM_RES;
        const double sp = res[RES_SP];
        const double wgt = R.params[8] > 0 ? sp : 1.0 - sp;
        // F1 + w (F2 - F1) in the fixed point of the force sums, w in units of 2^-32
        // (w in [0, 1]: at most 2^32; its rounding is 2^-33 relative to F2 - F1),
        // the product by a 128-bit multiply (floor), then one conversion per
        // component and the exact 2^-32 scaling in the exponent field
        const long long w32 = __double2ll_rn(wgt * 4294967296.0);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const long long f1 = (long long)a.F[(size_t)k * a.NA + s];
            const long long f2 = (long long)a.F[(size_t)(3 + k) * a.NA + s];
            const long long d = a.full ? f2 - f1 : f2;
            const long long hi = __mul64hi(d, w32);
            const unsigned long long lo = (unsigned long long)d * (unsigned long long)w32;
            const long long v = f1 + (long long)(((unsigned long long)hi << 32) | (lo >> 32));
            f[k] = R.var_nb ? fix_scaled(v) : 0.0;
            if (a.f_nb) a.f_nb[3 * (size_t)g + k] = fix_scaled(f1);
        }
    }
    const int g0 = g - lane;  // the warp's first atom
    const int nv = min(32, a.n_in - g0);
    if (nv <= 0) return;
    double* const dst = fo + 3 * (size_t)g0;
    if (nv == 32 && (reinterpret_cast<size_t>(dst) & 15) == 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) s_f[w][3 * lane + k] = f[k];
        __syncwarp();
        const double2* src = reinterpret_cast<const double2*>(s_f[w]);
        double2* d2 = reinterpret_cast<double2*>(dst);
        d2[lane] = src[lane];
        if (lane < 16) d2[32 + lane] = src[32 + lane];
    } else if (lane < nv) {
#pragma unroll
        for (int k = 0; k < 3; k++) dst[3 * lane + k] = f[k];
    }
}

void launch_output(const Args& a, cudaStream_t s) {
    k_output<<<(a.n_in + kOutThreads - 1) / kOutThreads, kOutThreads, 0, s>>>(a);
}

// replicas x states energy matrix: beta * (e0(r; dir_s) + W_s(usc_s(u(r; dir_s))))
__global__ void k_matrix(Args a) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.R * a.R) return;
    int r = idx / a.R, s = idx % a.R;
    const double* res = a.results + (size_t)r * NUM_RES;
    double out[NUM_RES];
    bool v = a.reps[r].var_nb;
    atm_merge(v ? res[RES_E1] : 0.0, v ? res[RES_E2] : 0.0, a.reps[s].params, out);
    a.matrix[idx] = *a.beta * out[RES_ENERGY];
}

void launch_matrix(const Args& a, cudaStream_t s) {
    int n = a.R * a.R;
    k_matrix<<<(n + 127) / 128, 128, 0, s>>>(a);
}

// Backward pass of L = sum_r g_r W_r from the last (adjoint) evaluation.  With
// s = +1 for direction > 0 (u = U2 - U1) and -1 otherwise:
//   dW/dx = -s W'(u) (F2 - F1),  dW/dd = -s W'(u) F2,
//   dW/d{q, sigma, eps} = s W'(u) d(U2 - U1)/d{q, sigma, eps}.
__global__ void k_adjoint(Args a, const double* g, double* dx, double* dd, double* dq, double* dsig, double* deps,
                          double* dpar) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < a.R * 5 && dpar) {
        const int r = s / 5, k = s % 5;
        dpar[s] = g[r] * a.results[(size_t)r * NUM_RES + RES_DL1 + k];
    }
    if (s >= a.NA) return;
    const int o = a.orig[s];
    if (o < 0) return;
    const int rep = a.block_rep[s >> 5];
    const RepDev& R = a.reps[rep];
    const double* res = a.results + (size_t)rep * NUM_RES;
    const double sgn = R.params[8] > 0 ? 1.0 : -1.0;
    const double w = R.var_nb ? g[rep] * res[RES_DWDU] : 0.0;
    const size_t u = (size_t)(R.in_off + o);
    const double sc = 1.0 / kFixScale;
    for (int k = 0; k < 3; k++) {
        const long long f1 = (long long)a.F[(size_t)k * a.NA + s];
        const long long f2 = (long long)a.F[(size_t)(3 + k) * a.NA + s];
        const double delta = a.full ? (double)(f2 - f1) : (double)f2;  // F2 - F1
        if (dx) dx[3 * u + k] = -sgn * w * delta * sc;
        if (dd) dd[3 * u + k] = -sgn * w * ((double)f1 + delta) * sc;
    }
    if (a.adjoint) {
        const double dqs = (double)(long long)a.D[s] * sc;
        if (dq) dq[u] = sgn * w * dqs * (double)a.sqrt_ke;
        if (dsig) dsig[u] = sgn * w * (double)(long long)a.D[a.NA + s] * sc;
        if (deps) deps[u] = sgn * w * (double)(long long)a.D[2 * (size_t)a.NA + s] * sc;
    }
}

void launch_adjoint(const Args& a, const double* g, double* dx, double* dd, double* dq, double* dsig, double* deps,
                    double* dpar, cudaStream_t s) {
    int n = a.NA > 5 * a.R ? a.NA : 5 * a.R;
    k_adjoint<<<(n + 255) / 256, 256, 0, s>>>(a, g, dx, dd, dq, dsig, deps, dpar);
}

}  // namespace atm
