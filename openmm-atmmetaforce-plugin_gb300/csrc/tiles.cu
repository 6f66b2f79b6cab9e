// Pair-tile lists and the pair-tile kernel (direct-space LJ + reaction field /
// Ewald) of the ATM evaluation path, sm_103a.
//
// A "row" is one 32-atom block I at one geometry (state 1, state 2, or one of the
// two geometries of the ligand-difference tiles); its candidate blocks may be split
// over several rows (parts) when rows are few.  Tiles are half blocks: 16 i atoms
// (I16 = 2 I or 2 I + 1) by 16 j slots.  k_find builds, per row:
//   - exclusion sub-tiles: the 16 x 16 sub-tiles with a computed pair of the
//     diagonal tile and of every block pair holding an exclusion, with masks;
//   - atom tiles: the atoms j of every other candidate block J (bounding boxes
//     closer than the cutoff) that lie within the cutoff of block I's bounding
//     box and then within the cutoff of at least one atom of a half block, packed
//     16 per tile of that half;
//   - an even number of tiles (an empty atom tile fills an odd count), so that the
//     two halves of a warp in the pair-tile kernel always hold tiles of one row.
// The per-atom tests remove most of the pair slots a block tile would spend beyond
// the cutoff.
//
// Tile entry (int4):
//   x = I16
//   y = J16 (exclusion sub-tiles)
//   z = row | kind << 28 | atom_tile << 30
//   w = aux | slot << 20 | pbc << 31
//       aux  = mask id + 1 (sub-tiles) or number of valid j (atom tiles, 0: filler)
//       slot = position of the tile within its row (energy slot)
//       pbc  = 1 when every pair needs its own minimum image (small boxes)
#include <algorithm>

#include <cuda_fp16.h>

#include "kernels.cuh"

namespace atm {

#define FULL_MASK 0xffffffffu

constexpr int kFindWarps = 4;
constexpr int kTileGrab = 4;  // tiles per grab of the pair-tile kernel

__device__ __forceinline__ void fix_add_t(unsigned long long* p, float v) {
    atomicAdd(p, fix_bits(v));
}

// Compensated FP32 sum (Knuth's TwoSum): s + c carries the exact sum of the
// terms to a relative error of order 2^-48 of their magnitudes, with FP32
// instructions only (FP64 arithmetic is 1/64 of the FP32 rate on this part).
__device__ __forceinline__ void two_sum_add(float& s, float& c, float x) {
    const float t = s + x;
    const float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
}

// Asynchronous global -> shared copies (cp.async), which hold no registers
// while they are in flight; a warp waits for its own and then __syncwarp()s.
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// The box of a replica in registers, for minimum images in the pair loops.
struct ImgBox {
    float Lx, Ly, Lz, iLx, iLy, iLz, bx, cx, cy;
    int tric;
};
__device__ __forceinline__ ImgBox img_box(const RepDev& R) {
    return ImgBox{R.box[0], R.box[1], R.box[2], R.ibox[0], R.ibox[1], R.ibox[2], R.tilt[0], R.tilt[1], R.tilt[2],
                  R.tric};
}
// OpenMM's minimum image (reduced triclinic box: c, then b, then a; per axis
// when orthorhombic)
__device__ __forceinline__ void min_image_b(float& x, float& y, float& z, const ImgBox& B) {
    if (B.tric) {
        const float kz = rintf(z * B.iLz);
        x -= kz * B.cx;
        y -= kz * B.cy;
        z -= kz * B.Lz;
        const float ky = rintf(y * B.iLy);
        x -= ky * B.bx;
        y -= ky * B.Ly;
    } else {
        y -= B.Ly * rintf(y * B.iLy);
        z -= B.Lz * rintf(z * B.iLz);
    }
    x -= B.Lx * rintf(x * B.iLx);
}

// The finder's minimum image: its orthorhombic instantiation (no replica of the
// batch is triclinic) keeps only the per-axis form, and none of the tilts.
// (The box is read from the replica's table where it is used: held in registers
// across a row it costs the finder spills.)
template <bool TRIC>
__device__ __forceinline__ void min_image_t(float& x, float& y, float& z, const RepDev& R) {
    if constexpr (TRIC) {
        min_image3(x, y, z, R);
    } else {
        x -= R.box[0] * rintf(x * R.ibox[0]);
        y -= R.box[1] * rintf(y * R.ibox[1]);
        z -= R.box[2] * rintf(z * R.ibox[2]);
    }
}

__device__ __forceinline__ float box_gap2(float dx, float dy, float dz, float hx, float hy, float hz) {
    dx = fmaxf(0.f, fabsf(dx) - hx);
    dy = fmaxf(0.f, fabsf(dy) - hy);
    dz = fmaxf(0.f, fabsf(dz) - hz);
    return dx * dx + dy * dy + dz * dz;
}

// Are two blocks' bounding boxes closer than the cutoff?  The centres' minimum
// image (per axis, exact for orthorhombic boxes); triclinic rows that need
// per-pair images (all_images) take the closest of the 125 images around it.
template <bool TRIC>
__device__ __forceinline__ bool boxes_close(float4 ci, float4 hi, float4 cj, float4 hj, const RepDev& R, float rc2,
                                            bool all_images = false) {
    float dx = cj.x - ci.x, dy = cj.y - ci.y, dz = cj.z - ci.z;
    min_image_t<TRIC>(dx, dy, dz, R);
    const float hx = hi.x + hj.x, hy = hi.y + hj.y, hz = hi.z + hj.z;
    if (!TRIC || !all_images) return box_gap2(dx, dy, dz, hx, hy, hz) < rc2;
    for (int k = -2; k <= 2; k++)
        for (int j = -2; j <= 2; j++)
            for (int i = -2; i <= 2; i++) {
                const float vx = dx + i * R.box[0] + j * R.tilt[0] + k * R.tilt[1];
                const float vy = dy + j * R.box[1] + k * R.tilt[2];
                const float vz = dz + k * R.box[2];
                if (box_gap2(vx, vy, vz, hx, hy, hz) < rc2) return true;
            }
    return false;
}

// Is atom p within the cutoff of the box of block I (minimum image of the offset
// from the box centre)?
template <bool TRIC>
__device__ __forceinline__ bool point_close(float4 ci, float4 hi, float4 p, const RepDev& R, float rc2) {
    float dx = p.x - ci.x, dy = p.y - ci.y, dz = p.z - ci.z;
    min_image_t<TRIC>(dx, dy, dz, R);
    return box_gap2(dx, dy, dz, hi.x, hi.y, hi.z) < rc2;
}

// Centre and half extent of block I at the geometry of a row.
__device__ __forceinline__ void row_box(const Args& a, int I, int kind, float4& c, float4& h) {
    if (kind == ROW_STATE2) {
        c = a.bb_c2[I];
        h = a.bb_h2[I];
    } else {
        c = a.bb_c[I];
        h = a.bb_h[I];
        if (kind == ROW_DIFF2) {
            float4 d = a.block_d[I];
            c.x += d.x;
            c.y += d.y;
            c.z += d.z;
        }
    }
}

constexpr int kStageAtoms = 2048;  // culled atoms staged in shared memory per row

// Position of slot s at the geometry of a row kind, as the pair-tile kernel reads it.
__device__ __forceinline__ float4 row_pos(const Args& a, int kind, int s) {
    float4 p = (kind == ROW_STATE2 ? a.posq2 : a.posq)[s];
    if (kind == ROW_DIFF2) {
        const float4 d = a.displ[s];
        p.x += d.x;
        p.y += d.y;
        p.z += d.z;
    }
    return p;
}

// Positions of the atoms of block I at the geometry of a row, taken to the
// periodic image nearest the box centre (as the pair-tile kernel does), into the
// warp's shared memory for the exact cut: FP32 (absolute), or with hcut the
// offsets from the box centre as half2 pairs (atoms 2m, 2m+1: x, y, z; 16 bytes
// per pair, in the first half of the same buffer).
template <bool TRIC>
__device__ __forceinline__ void load_ipos(const Args& a, const RepDev& R, int I, int kind, float4 ci, int lane,
                                          float4* s_ipos, bool hcut) {
    const float4 pi = row_pos(a, kind, I * kTile + lane);
    float rx = pi.x - ci.x, ry = pi.y - ci.y, rz = pi.z - ci.z;
    min_image_t<TRIC>(rx, ry, rz, R);
    if (hcut) {
        const float nx = __shfl_down_sync(FULL_MASK, rx, 1), ny = __shfl_down_sync(FULL_MASK, ry, 1),
                    nz = __shfl_down_sync(FULL_MASK, rz, 1);
        if ((lane & 1) == 0) {
            const __half2 hx = __floats2half2_rn(rx, nx), hy = __floats2half2_rn(ry, ny), hz = __floats2half2_rn(rz, nz);
            uint4 q;
            q.x = *reinterpret_cast<const unsigned*>(&hx);
            q.y = *reinterpret_cast<const unsigned*>(&hy);
            q.z = *reinterpret_cast<const unsigned*>(&hz);
            q.w = 0u;
            reinterpret_cast<uint4*>(s_ipos)[lane >> 1] = q;
        }
    } else {
        s_ipos[lane] = make_float4(ci.x + rx, ci.y + ry, ci.z + rz, pi.w);
    }
    __syncwarp();
}

// Rows whose block box is at most kHalfCutMaxH (nm) in every dimension, with a
// cutoff of at most kHalfCutMaxRc, take the half-precision exact cut.  Offsets
// from the box centre are then below 2.25 nm (rounded by <= 2^-10 nm) and a pair
// near the cutoff has |dx| <= 1.5 nm per component, so each component of the
// half difference is off by <= 0.0017 nm and r^2 by <= 0.0117 nm^2 with the
// roundings of the products: r by <= 0.004 nm.  The cut distance is widened by
// kHalfCutMargin, so no pair within the cutoff of the FP32 kernel is lost.
constexpr float kHalfCutMaxH = 0.75f, kHalfCutMaxRc = 1.5f, kHalfCutMargin = 0.005f;

// Second cut of staged atoms list[from, natom): keeps the atoms j within the
// cutoff of at least one atom of block I (the box test keeps every atom within
// the cutoff of the box, corners included), flagged by half block: bit 30 within
// the cutoff of an atom 0..15 of I, bit 31 of an atom 16..31 (the pair tiles are
// half blocks).  Positions are taken to the periodic image nearest the box
// centre, as the pair-tile kernel does; the threshold is widened by 1e-5 so that
// no pair the kernel counts can be dropped by rounding.  In place, order kept;
// returns from + the number kept.
constexpr unsigned kHalfA = 1u << 30, kHalfB = 1u << 31, kSlotBits = kHalfA - 1u;

template <bool TRIC>
__device__ __forceinline__ int exact_cut_half(const Args& a, const RepDev& R, int kind, float4 ci, int lane,
                                              int* list, int from, int natom, const float4* s_ipos) {
    const float rcm = sqrtf(a.rcl2) + kHalfCutMargin;
    const __half2 thr = __float2half2_rn(rcm * rcm);
    const uint4* ih = reinterpret_cast<const uint4*>(s_ipos);
    int kept = from;
    for (int g = from; g < natom; g += 32) {
        const int k = g + lane;
        const bool valid = k < natom;
        const int j = valid ? list[k] : 0;
        float rx = 64.f, ry = 64.f, rz = 64.f;  // invalid lanes never hit
        if (valid) {
            const float4 p = row_pos(a, kind, j);
            rx = p.x - ci.x;
            ry = p.y - ci.y;
            rz = p.z - ci.z;
            min_image_t<TRIC>(rx, ry, rz, R);
        }
        const __half2 hx = __float2half2_rn(rx), hy = __float2half2_rn(ry), hz = __float2half2_rn(rz);
        bool hitA = false, hitB = false;
        // two i atoms per instruction, eight per step; each half until every lane has decided it
        for (int m0 = 0; m0 < kHalf / 2; m0 += 4) {
#pragma unroll
            for (int m = m0; m < m0 + 4; m++) {
                const uint4 q = ih[m];
                const __half2 dx = __hsub2(hx, *reinterpret_cast<const __half2*>(&q.x));
                const __half2 dy = __hsub2(hy, *reinterpret_cast<const __half2*>(&q.y));
                const __half2 dz = __hsub2(hz, *reinterpret_cast<const __half2*>(&q.z));
                const __half2 r2 = __hfma2(dx, dx, __hfma2(dy, dy, __hmul2(dz, dz)));
                hitA |= !__hbge2(r2, thr);  // either atom of the pair within the widened cutoff
            }
            if (__all_sync(FULL_MASK, hitA || !valid)) break;
        }
        for (int m0 = kHalf / 2; m0 < kHalf; m0 += 4) {
#pragma unroll
            for (int m = m0; m < m0 + 4; m++) {
                const uint4 q = ih[m];
                const __half2 dx = __hsub2(hx, *reinterpret_cast<const __half2*>(&q.x));
                const __half2 dy = __hsub2(hy, *reinterpret_cast<const __half2*>(&q.y));
                const __half2 dz = __hsub2(hz, *reinterpret_cast<const __half2*>(&q.z));
                const __half2 r2 = __hfma2(dx, dx, __hfma2(dy, dy, __hmul2(dz, dz)));
                hitB |= !__hbge2(r2, thr);
            }
            if (__all_sync(FULL_MASK, hitB || !valid)) break;
        }
        __syncwarp();
        const bool keep = valid && (hitA || hitB);
        const unsigned b = __ballot_sync(FULL_MASK, keep);
        if (keep)
            list[kept + __popc(b & ((1u << lane) - 1u))] =
                (int)((unsigned)j | (hitA ? kHalfA : 0u) | (hitB ? kHalfB : 0u));
        kept += __popc(b);
        __syncwarp();
    }
    return kept;
}

template <bool TRIC>
__device__ __noinline__ int exact_cut(const Args& a, const RepDev& R, int kind, float4 ci, int lane, int* list,
                                         int from, int natom, const float4* s_ipos, bool hcut) {
    if (hcut) return exact_cut_half<TRIC>(a, R, kind, ci, lane, list, from, natom, s_ipos);
    const float rc2 = a.rcl2 * 1.00001f;
    int kept = from;
    for (int g = from; g < natom; g += 32) {
        const int k = g + lane;
        const bool valid = k < natom;
        const int j = valid ? list[k] : 0;
        bool hitA = false, hitB = false;
        float4 p = make_float4(1.0e15f, 1.0e15f, 1.0e15f, 0.f);  // invalid lanes never hit
        if (valid) {
            p = row_pos(a, kind, j);
            float rx = p.x - ci.x, ry = p.y - ci.y, rz = p.z - ci.z;
            min_image_t<TRIC>(rx, ry, rz, R);
            p.x = ci.x + rx;
            p.y = ci.y + ry;
            p.z = ci.z + rz;
        }
        // eight i atoms at a time; each half until every lane has decided it
        for (int q0 = 0; q0 < kHalf; q0 += 8) {
#pragma unroll
            for (int q = q0; q < q0 + 8; q++) {
                const float4 o = s_ipos[q];
                const float dx = p.x - o.x, dy = p.y - o.y, dz = p.z - o.z;
                hitA |= dx * dx + dy * dy + dz * dz < rc2;
            }
            if (__all_sync(FULL_MASK, hitA || !valid)) break;
        }
        for (int q0 = kHalf; q0 < 32; q0 += 8) {
#pragma unroll
            for (int q = q0; q < q0 + 8; q++) {
                const float4 o = s_ipos[q];
                const float dx = p.x - o.x, dy = p.y - o.y, dz = p.z - o.z;
                hitB |= dx * dx + dy * dy + dz * dz < rc2;
            }
            if (__all_sync(FULL_MASK, hitB || !valid)) break;
        }
        __syncwarp();
        const bool keep = valid && (hitA || hitB);
        const unsigned b = __ballot_sync(FULL_MASK, keep);
        if (keep)
            list[kept + __popc(b & ((1u << lane) - 1u))] =
                (int)((unsigned)j | (hitA ? kHalfA : 0u) | (hitB ? kHalfB : 0u));
        kept += __popc(b);
        __syncwarp();
    }
    return kept;
}

// One pass over the candidate blocks of a row (bounding boxes closer than the
// cutoff, no exclusion with I) and their atoms within the cutoff of block I's
// box, written in a fixed order to consecutive j slots of out.
//   CUT = false: returns the number of atoms and writes the first cap of them.
//   CUT = true (out: the warp's stage in shared memory, s_ipos loaded): whenever
//     the stage nears cap, the exact cut thins the atoms staged since the last
//     cut; returns the number of atoms kept, or -1 when they do not fit (then
//     raw holds the number of atoms before any cut).
// The row's exclusion partners are held one per lane (rows with more than 32 fall
// back to reading the list), and four candidate blocks are loaded per step so
// that their latencies overlap.
template <bool CUT, bool TRIC>
__device__ __forceinline__ int row_atoms(const Args& a, const RepDev& R, int I, int kind, float4 ci, float4 hi,
                                         const int2* ee, int e0, int e1, int lane, int* out, int cap,
                                         const float4* s_ipos, int& raw, int first, int stride,
                                         bool hcut = false, bool all_images = false) {
    const bool diff = kind >= ROW_DIFF1;
    const bool g2 = kind == ROW_DIFF2;
    const int cls_i = a.block_cls[I];
    const float4* P = kind == ROW_STATE2 ? a.posq2 : a.posq;
    const float4* BH = kind == ROW_STATE2 ? a.bb_h2 : a.bb_h;
    const int nex = e1 - e0;
    const int my_ex = lane < nex ? ee[e0 + lane].x : -1;
    int natom = 0, cut_from = 0;
    bool over = false;
    raw = 0;
    const int jb = diff ? R.block_begin : I + 1;
    for (int base = jb + first; base < R.block_end; base += 32 * stride) {
        const int Jl = base + lane * stride;
        bool ok = Jl < R.block_end;
        if (ok && diff) {
            const int cj = a.block_cls[Jl];
            ok = Jl != I && cj != cls_i && (cj == 0 || cls_i < cj);
        }
        if (ok) {
            float4 cj4, hj4;
            if (kind == ROW_STATE2) {
                cj4 = a.bb_c2[Jl];
                hj4 = a.bb_h2[Jl];
            } else {
                cj4 = a.bb_c[Jl];
                hj4 = a.bb_h[Jl];
                if (g2) {
                    const float4 dd = a.block_d[Jl];  // zero for blocks that do not move
                    cj4.x += dd.x;
                    cj4.y += dd.y;
                    cj4.z += dd.z;
                }
            }
            ok = boxes_close<TRIC>(ci, hi, cj4, hj4, R, a.rcl2, all_images);
            if (nex > 32)
                for (int k = e0; ok && k < e1; k++)
                    if (ee[k].x == Jl) ok = false;
        }
        if (nex <= 32) {
            // drop the exclusion partners: lane q holds partner q
            for (int q = 0; q < nex; q++) {
                const int xj = __shfl_sync(FULL_MASK, my_ex, q);
                if (xj == Jl) ok = false;
            }
        }
        unsigned cand = __ballot_sync(FULL_MASK, ok);
        while (cand) {
            int J[4], n[4];
            float4 p[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                J[t] = cand ? base + (__ffs(cand) - 1) * stride : -1;
                if (cand) cand &= cand - 1;
            }
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int jj = (J[t] >= 0 ? J[t] : J[0]) * kTile + lane;
                p[t] = P[jj];
                n[t] = J[t] >= 0 ? __float_as_int(BH[J[t]].w) : 0;
            }
            if (g2) {
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const float4 d = a.displ[(J[t] >= 0 ? J[t] : J[0]) * kTile + lane];
                    p[t].x += d.x;
                    p[t].y += d.y;
                    p[t].z += d.z;
                }
            }
#pragma unroll
            for (int t = 0; t < 4; t++) {
                // (triclinic rows with per-pair images keep every atom of a candidate block)
                const bool in = lane < n[t] && (all_images || point_close<TRIC>(ci, hi, p[t], R, a.rcl2));
                const unsigned b = __ballot_sync(FULL_MASK, in);
                const int k = natom + __popc(b & ((1u << lane) - 1u));
                if (in && k < cap && !over) out[k] = J[t] * kTile + lane;
                natom += __popc(b);
                raw += __popc(b);
            }
            if (CUT && !over && natom > cap - 4 * kTile) {
                __syncwarp();
                natom = exact_cut<TRIC>(a, R, kind, ci, lane, out, cut_from, min(natom, cap), s_ipos, hcut);
                cut_from = natom;
                over = natom > cap - 4 * kTile;
            }
        }
    }
    if (CUT) {
        if (over) return -1;
        __syncwarp();
        natom = exact_cut<TRIC>(a, R, kind, ci, lane, out, cut_from, natom, s_ipos, hcut);
    }
    return natom;
}

// The tiles of one row (one warp; stage and ipos: the warp's shared memory).
template <bool TRIC>
__device__ __forceinline__ void find_row(const Args& a, int row, int lane, int* stage, float4* ipos) {
    const int4 d = a.row_desc[row];
    const int I = d.x, kind = d.y;
    // part `part` of `nparts`: the candidate blocks J = first + part + k nparts;
    // part 0 also holds the block tiles
    const int part = d.w & 0xff, nparts = max(1, d.w >> 8);
    const RepDev& R = a.reps[d.z];
    const bool diff = kind >= ROW_DIFF1;
    const int* es = diff ? a.dx_start : a.ex_start;
    const int2* ee = diff ? a.dx_ent : a.ex_ent;
    const int e0 = es[I], e1 = es[I + 1];
    float4 ci, hi;
    row_box(a, I, kind, ci, hi);
    // pbc: some pair of an atom tile may need its own minimum image when the
    // cutoff sphere around block I reaches half a box length (at the list cutoff:
    // while the lists are kept, a block's box grows by up to skin / 2 per side)
    const float rc = sqrtf(a.rcl2);
    unsigned pbc;
    if (TRIC && R.tric) {
        // images are coupled across axes: the centres' minimum image is the one of
        // every pair when rc plus both blocks' half extents (the replica's largest
        // for J) stays below half the smallest face distance
        const float hn = sqrtf(hi.x * hi.x + hi.y * hi.y + hi.z * hi.z);
        pbc = rc + hn + __uint_as_float(a.rep_hmax[d.z]) >= 0.5f * R.wmin ? 1u : 0u;
    } else {
        pbc = (rc + 2.f * hi.x >= 0.5f * R.box[0] || rc + 2.f * hi.y >= 0.5f * R.box[1] ||
               rc + 2.f * hi.z >= 0.5f * R.box[2])
                  ? 1u
                  : 0u;
    }
    const bool all_images = TRIC && pbc && R.tric;
    // staged in shared memory and cut there; rows whose atoms do not fit, and rows
    // that need per-pair images (no exact cut), are written by a second pass
    int raw = 0, natom = -1;
    if (!pbc) {
        const bool hcut = rc <= kHalfCutMaxRc && fmaxf(hi.x, fmaxf(hi.y, hi.z)) <= kHalfCutMaxH;
        load_ipos<TRIC>(a, R, I, kind, ci, lane, ipos, hcut);
        natom = row_atoms<true, TRIC>(a, R, I, kind, ci, hi, ee, e0, e1, lane, stage, kStageAtoms, ipos, raw, part,
                                nparts, hcut);
    } else {
        natom = row_atoms<false, TRIC>(a, R, I, kind, ci, hi, ee, e0, e1, lane, stage, kStageAtoms, ipos, raw, part,
                                 nparts, false, all_images);
        if (natom > kStageAtoms) natom = -1;
    }
    __syncwarp();
    const bool staged = natom >= 0;
    const bool flagged = staged && !pbc;  // cut atoms carry their half-block flags
    if (!staged) natom = raw;
    int nA = natom, nB = natom;  // uncut atoms go to both halves
    if (flagged) {
        nA = nB = 0;
        for (int k = lane; k < natom; k += 32) {
            const unsigned v = (unsigned)stage[k];
            nA += (v & kHalfA) ? 1 : 0;
            nB += (v & kHalfB) ? 1 : 0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            nA += __shfl_xor_sync(FULL_MASK, nA, o);
            nB += __shfl_xor_sync(FULL_MASK, nB, o);
        }
    }
    // half-block tiles: the exclusion sub-tiles (part 0), then the atom tiles of
    // each half; an even count, so that the two halves of a warp share a row
    const int* ss = diff ? a.dxs_start : a.exs_start;
    const int4* se = diff ? a.dxs_ent : a.exs_ent;
    const int s0 = ss[I];
    const int nblock = part == 0 ? ss[I + 1] - s0 : 0;
    const int nta = (nA + kHalf - 1) / kHalf, ntb = (nB + kHalf - 1) / kHalf;
    int n = nblock + nta + ntb;
    const bool filler = n & 1;
    n += filler ? 1 : 0;
    if (lane == 0) atomicMax(&a.status->max_row, n);
    if (n > a.row_cap) {
        if (lane == 0) atomicOr(&a.status->overflow, 2);
        n = 0;  // the evaluation is repeated with larger buffers
    }
    int tbase = 0;
    if (lane == 0) tbase = atomicAdd(&a.status->tile_count, n);
    tbase = __shfl_sync(FULL_MASK, tbase, 0);
    if (lane == 0) {
        a.row_count[row] = n;
        a.row_tbase[row] = tbase;
    }
    if (n == 0) return;
    if (tbase + n > a.tile_cap) {
        if (lane == 0) atomicOr(&a.status->overflow, 1);
        return;
    }
    int* outA = a.tile_j + (size_t)(tbase + nblock) * kHalf;
    int* outB = outA + (size_t)nta * kHalf;
    if (flagged) {
        int ka = 0, kb = 0;
        for (int g = 0; g < natom; g += 32) {
            const int k = g + lane;
            const unsigned v = k < natom ? (unsigned)stage[k] : 0u;
            const bool fa = v & kHalfA, fb = v & kHalfB;
            const unsigned ba = __ballot_sync(FULL_MASK, fa), bb = __ballot_sync(FULL_MASK, fb);
            const unsigned lt = (1u << lane) - 1u;
            if (fa) outA[ka + __popc(ba & lt)] = (int)(v & kSlotBits);
            if (fb) outB[kb + __popc(bb & lt)] = (int)(v & kSlotBits);
            ka += __popc(ba);
            kb += __popc(bb);
        }
    } else if (staged) {
        for (int k = lane; k < natom; k += 32) {
            outA[k] = stage[k];
            outB[k] = stage[k];
        }
    } else {
        // second pass: the same atoms, in the same order, straight into the j slots of both halves
        row_atoms<false, TRIC>(a, R, I, kind, ci, hi, ee, e0, e1, lane, outA, natom, ipos, raw, part, nparts, false,
                         all_images);
        row_atoms<false, TRIC>(a, R, I, kind, ci, hi, ee, e0, e1, lane, outB, natom, ipos, raw, part, nparts, false,
                         all_images);
    }
    for (int k = nA + lane; k < kHalf * nta; k += 32) outA[k] = -1;
    for (int k = nB + lane; k < kHalf * ntb; k += 32) outB[k] = -1;
    const int zword = row | (kind << 28);
    for (int k = lane; k < nblock; k += 32) {
        const int4 e = se[s0 + k];
        a.tiles[tbase + k] = make_int4(e.x, e.y, zword, (int)((unsigned)(e.z + 1) | ((unsigned)k << 20) | (pbc << 31)));
    }
    for (int k = lane; k < nta + ntb; k += 32) {
        const bool hb = k >= nta;
        const int kk = hb ? k - nta : k;
        const int cnt = min(kHalf, (hb ? nB : nA) - kHalf * kk);
        a.tiles[tbase + nblock + k] = make_int4(2 * I + (hb ? 1 : 0), 0, zword | (1 << 30),
                                                (int)((unsigned)cnt | ((unsigned)(nblock + k) << 20) | (pbc << 31)));
    }
    if (filler && lane == 0)  // an empty atom tile (no j), energy slot n - 1
        a.tiles[tbase + n - 1] = make_int4(2 * I, 0, zword | (1 << 30), (int)((unsigned)(n - 1) << 20));
}

// Persistent: every warp takes rows from a counter, last rows first (the
// state-2 / difference rows at the end of the row list scan every block of
// their replica and are the longest, so they start early); the next row is
// requested before the current one is built.
template <bool TRIC>
__global__ void __launch_bounds__(kFindWarps * 32, 6) k_find(Args a) {
    __shared__ int s_stage[kFindWarps][kStageAtoms];
    __shared__ float4 s_ipos[kFindWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (!a.status->rebuild) return;  // the lists of an earlier evaluation still hold
    if (a.skin_half2 > 0.f)  // the positions of this build, for the displacement test
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.NA; s += gridDim.x * blockDim.x)
            a.posq_ref[s] = a.posq[s];
    // the first row of every warp is fixed, the later ones come from the counter
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int mine = a.nrows;
    while (k < a.nrows) {
        if (lane == 0) mine = nw < a.nrows ? nw + atomicAdd(&a.status->next_row, 1) : a.nrows;
        find_row<TRIC>(a, a.nrows - 1 - k, lane, s_stage[w], s_ipos[w]);
        __syncwarp();
        k = __shfl_sync(FULL_MASK, mine, 0);
    }
}

int find_warps_per_sm() {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_find<true>, kFindWarps * 32, 0);
    return std::max(1, per_sm) * kFindWarps;
}

void launch_find(const Args& a, cudaStream_t s) {
    static int per_sm = 0, sms = 0;
    if (per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_find<true>, kFindWarps * 32, 0);
        if (per_sm < 1) per_sm = 1;
    }
    const int blocks = std::min(per_sm * sms, (a.nrows + kFindWarps - 1) / kFindWarps);
    if (a.any_tric)
        k_find<true><<<blocks, kFindWarps * 32, 0, s>>>(a);
    else
        k_find<false><<<blocks, kFindWarps * 32, 0, s>>>(a);
}

// The hardware approximations of the PTX ISA with subnormal inputs and results
// flushed to zero (no pair term produces or uses a subnormal value that matters),
// which spares the instructions that handle subnormals around each one.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_ftz(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kLog2e = 1.4426950408889634f;

// erfc(x) for x >= 0: Abramowitz & Stegun, Handbook of Mathematical Functions,
// eq. 7.1.26 (|error| <= 1.5e-7), sharing exp(-x^2) with the force term:
// erfc(x) = t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-x^2), t = 1 / (1 + p x).
constexpr float kErfcP = 0.3275911f;
constexpr float kErfcA1 = 0.254829592f, kErfcA2 = -0.284496736f, kErfcA3 = 1.421413741f,
                kErfcA4 = -1.453152027f, kErfcA5 = 1.061405429f;
__device__ __forceinline__ float erfc_as(float x, float expmx2) {
    const float t = rcp_ftz(1.0f + kErfcP * x);
    const float p = t * (kErfcA1 + t * (kErfcA2 + t * (kErfcA3 + t * (kErfcA4 + t * kErfcA5))));
    return p * expmx2;
}

// Energy e and fr = -(dE/dr)/r of one pair (q already scaled by sqrt(k_e),
// eps4 = 4 sqrt(eps_i eps_j), sig = (sigma_i + sigma_j)/2).
template <int METHOD>
__device__ __forceinline__ void pair_eval(float r2, float qq, float sig, float eps4, float alpha, float krf, float crf,
                                          float& e, float& fr) {
    const float invr = rsqrt_ftz(r2);
    const float invr2 = invr * invr;
    const float s2 = sig * sig * invr2;
    const float s6 = s2 * s2 * s2;
    const float t6 = eps4 * s6;
    e = t6 * s6 - t6;
    if (METHOD == 4) {
        const float ex = ex2_ftz(r2 * (-alpha * alpha * kLog2e));  // exp(-alpha^2 r^2)
        // erfc(alpha r) as in erfc_as, with the constant folded into alpha
        const float t = rcp_ftz(fmaf(0.3275911f * alpha, r2 * invr, 1.0f));
        const float ec =
            t * (0.254829592f + t * (-0.284496736f + t * (1.421413741f + t * (-1.453152027f + t * 1.061405429f)))) *
            ex * invr;
        e += qq * ec;
        fr = fmaf(t6, fmaf(12.0f, s6, -6.0f), qq * (ec + 1.1283791670955126f * alpha * ex)) * invr2;
    } else {
        fr = (12.0f * t6 * s6 - 6.0f * t6) * invr2;
        e += qq * (invr + krf * r2 - crf);
        fr += qq * (invr * invr2 - 2.0f * krf);
    }
}

// The 16 steps of one half-block tile, on each half of the warp: lane l of a
// half meets j-slot (l+k)&15 at step k; j data are read from shared memory
// (stored twice over, so that slot (l+k)&15 is entry l+k of the lane's own base:
// a constant offset per unrolled step), j forces travel with their slot by
// shuffles within the half.  MASKED: a per-lane bit mask of the pairs to
// count (exclusions, padding); unmasked tiles park their padding j slots far away.
template <int METHOD, bool PBC, bool DIFF, bool MASKED>
__device__ __forceinline__ void tile_steps(const float4* __restrict__ sp, const float2* __restrict__ sl, float4 pi,
                                           float2 li, unsigned mask, int lane, const ImgBox& B, float rc2,
                                           float alpha, float krf, float crf, float3& fi, float3& fj, float& e32,
                                           float2& ec) {
    const int src = (lane & kHalf) | ((lane + 1) & (kHalf - 1));  // next lane of this half
    // the unmasked atom tiles carry most pairs; the other variants stay compact
    // so that the hot loop keeps the instruction cache
    constexpr int kUnroll = (!PBC && !DIFF) ? (MASKED ? 4 : 8) : 2;
#pragma unroll kUnroll
    for (int k = 0; k < kHalf; k++) {
        const float4 pj = sp[k];
        const float2 lj = sl[k];
        float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        if (PBC) min_image_b(dx, dy, dz, B);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const bool inc = MASKED ? (((mask >> k) & 1u) && r2 < rc2) : r2 < rc2;
        float e, fr;
        if (METHOD == 4) {
            // a pair not counted is evaluated at r^2 = 1e30 nm^2, where every term
            // comes out exactly zero (r^-6 and exp(-a^2 r^2) underflow; no overflow)
            pair_eval<METHOD>(inc ? r2 : 1.0e30f, pi.w * pj.w, li.x + lj.x, li.y * lj.y, alpha, krf, crf, e, fr);
        } else {
            pair_eval<METHOD>(inc ? r2 : 1.0f, pi.w * pj.w, li.x + lj.x, li.y * lj.y, alpha, krf, crf, e, fr);
            e = inc ? e : 0.0f;
            fr = inc ? fr : 0.0f;
        }
        if (DIFF) two_sum_add(ec.x, ec.y, e);
        else e32 += e;
        fi.x = fmaf(-fr, dx, fi.x);
        fi.y = fmaf(-fr, dy, fi.y);
        fi.z = fmaf(-fr, dz, fi.z);
        fj.x = __shfl_sync(FULL_MASK, fmaf(fr, dx, fj.x), src);
        fj.y = __shfl_sync(FULL_MASK, fmaf(fr, dy, fj.y), src);
        fj.z = __shfl_sync(FULL_MASK, fmaf(fr, dz, fj.z), src);
    }
}

// Two FP32 values in one 64-bit register pair, for the packed FP32 instructions
// of the sm_100 family (add / mul / fma .rn.f32x2: one instruction, two lanes of
// arithmetic, each rounded exactly as its scalar form).  lo = first, hi = second.
typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2_pack(float lo, float hi) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float f2_lo(f2x v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return lo;
}
__device__ __forceinline__ float f2_hi(f2x v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return hi;
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c) {
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b) {
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_add(f2x a, f2x b) {
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b) {
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_splat(float v) { return f2_pack(v, v); }

// Entries of the packed j layout of one half tile: entry m (0..15) holds j-slots
// m & 7 and (m & 7) + 8 side by side, as three 16-byte words
// {x, x', y, y'}, {z, z', q, q'}, {s, s', e, e'} (s = sigma/2, e = 2 sqrt(eps)).
constexpr int kPackedWords = 3;

// Lane l of a half (its j-slot data pj, lj) writes its slot into the two entries
// that carry it (entries l & 7 and (l & 7) + 8, component l >= 8).
// The PME variant stores the j charge times the erfc polynomial's leading
// coefficient (kPackedChargeScale), which its monic polynomial leaves out.
template <int METHOD>
constexpr float kPackedChargeScale = METHOD == 4 ? kErfcA5 : 1.0f;

template <int METHOD>
__device__ __forceinline__ void store_packed_j(float4* se, int l, float4 pj, float2 lj) {
    const int c = l >> 3;
    float* e0 = reinterpret_cast<float*>(se + kPackedWords * (l & 7));
    float* e1 = reinterpret_cast<float*>(se + kPackedWords * ((l & 7) + 8));
    const float v[6] = {pj.x, pj.y, pj.z, pj.w * kPackedChargeScale<METHOD>, lj.x, lj.y};
#pragma unroll
    for (int q = 0; q < 6; q++) {
        e0[2 * q + c] = v[q];
        e1[2 * q + c] = v[q];
    }
}

// The hot tile variant (atom tiles of state rows, no per-pair images, no mask:
// padding j slots parked far away) with two pairs per instruction: lane l of a
// half meets j-slots e = (l + k) & 7 and e + 8 at step k (8 steps, entry
// (l & 7) + k of the packed layout: a constant offset per unrolled step).  Within
// each group of 8 lanes of a half the j-force sums travel with their entry by
// shuffles; after the 8 steps lane l holds entry l & 7, and the two groups' sums
// of that entry are added, so that lane l returns the j force of its own slot l.
//   MASKED: smask holds, per j-slot s (bit s), whether the pair (this lane's i,
//   slot s) is counted (exclusion sub-tiles; excluded pairs, self pairs included,
//   are evaluated at r^2 = 1e30 like pairs beyond the cutoff).
template <int METHOD, bool MASKED>
__device__ __forceinline__ void tile_steps_x2(const float4* __restrict__ se, float4 pi, float2 li, int lane,
                                              unsigned smask, float rc2, float alpha, float krf, float crf,
                                              float3& fi, float3& fj, float& e32) {
    const int src = (lane & ~7) | ((lane + 1) & 7);  // next lane of this group of 8
    const f2x px = f2_splat(pi.x), py = f2_splat(pi.y), pz = f2_splat(pi.z), pq = f2_splat(pi.w);
    const f2x ps = f2_splat(li.x), pe = f2_splat(li.y);
    f2x fix = 0ull, fiy = 0ull, fiz = 0ull, fjx = 0ull, fjy = 0ull, fjz = 0ull, eacc = 0ull;
    const float4* base = se + kPackedWords * (lane & 7);
#pragma unroll 4
    for (int k = 0; k < 8; k++) {
        const ulonglong2 w0 = *reinterpret_cast<const ulonglong2*>(base + kPackedWords * k);
        const ulonglong2 w1 = *reinterpret_cast<const ulonglong2*>(base + kPackedWords * k + 1);
        const ulonglong2 w2 = *reinterpret_cast<const ulonglong2*>(base + kPackedWords * k + 2);
        const f2x dx = f2_sub(w0.x, px), dy = f2_sub(w0.y, py), dz = f2_sub(w1.x, pz);
        const f2x r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_mul(dz, dz)));
        const float ra = f2_lo(r2), rb = f2_hi(r2);
        bool ia = ra < rc2, ib = rb < rc2;
        if (MASKED) {
            const int sa = ((lane & 7) + k) & 7;  // slots sa and sa + 8 of this step
            ia = ia && ((smask >> sa) & 1u);
            ib = ib && ((smask >> (sa + 8)) & 1u);
        }
        const f2x qq = f2_mul(pq, w1.y), sig = f2_add(ps, w2.x), eps4 = f2_mul(pe, w2.y);
        f2x e, fr;
        if (METHOD == 4) {
            // a pair not counted is evaluated at r^2 = 1e30 nm^2, where every term is
            // exactly zero.  Written for few constant pairs (each costs two registers
            // in a loop budgeted at 64): t = 1 / (1 + c alpha r) as (1/r) / (1/r + c alpha),
            // the erfc polynomial monic (its leading coefficient a5 is carried by the
            // j charges of the packed layout, kPackedChargeScale), the LJ force as
            // 6 (E_lj + eps4 s^12).
            const f2x r2s = f2_pack(ia ? ra : 1.0e30f, ib ? rb : 1.0e30f);
            const f2x invr = f2_pack(rsqrt_ftz(f2_lo(r2s)), rsqrt_ftz(f2_hi(r2s)));
            const f2x invr2 = f2_mul(invr, invr);
            const f2x s2 = f2_mul(f2_mul(sig, sig), invr2);
            const f2x s6 = f2_mul(f2_mul(s2, s2), s2);
            const f2x t6 = f2_mul(eps4, s6);
            const f2x u6 = f2_mul(t6, s6);
            const f2x elj = f2_sub(u6, t6);
            const f2x flj = f2_add(u6, elj);  // (F_lj r^2) / 6
            const f2x xa = f2_mul(r2s, f2_splat(-alpha * alpha * kLog2e));
            const f2x ex = f2_pack(ex2_ftz(f2_lo(xa)), ex2_ftz(f2_hi(xa)));
            const f2x w = f2_add(invr, f2_splat(kErfcP * alpha));
            const f2x t = f2_mul(f2_pack(rcp_ftz(f2_lo(w)), rcp_ftz(f2_hi(w))), invr);
            f2x h = f2_add(t, f2_splat(kErfcA4 / kErfcA5));
            h = f2_fma(t, h, f2_splat(kErfcA3 / kErfcA5));
            h = f2_fma(t, h, f2_splat(kErfcA2 / kErfcA5));
            h = f2_fma(t, h, f2_splat(kErfcA1 / kErfcA5));
            const f2x bq = f2_mul(qq, ex);                      // a5 qq exp(-alpha^2 r^2)
            const f2x ec = f2_mul(bq, f2_mul(f2_mul(h, t), invr));  // qq erfc(alpha r) / r
            e = f2_add(ec, elj);
            const f2x fc = f2_fma(bq, f2_splat(1.1283791670955126f * alpha / kErfcA5), ec);
            fr = f2_mul(f2_fma(flj, f2_splat(6.0f), fc), invr2);
        } else {
            // reaction field: terms at r^2 (or 1 when not counted), then zeroed by the weight
            const f2x r2s = f2_pack(ia ? ra : 1.0f, ib ? rb : 1.0f);
            const f2x w = f2_pack(ia ? 1.0f : 0.0f, ib ? 1.0f : 0.0f);
            const f2x invr = f2_pack(rsqrt_ftz(f2_lo(r2s)), rsqrt_ftz(f2_hi(r2s)));
            const f2x invr2 = f2_mul(invr, invr);
            const f2x s2 = f2_mul(f2_mul(sig, sig), invr2);
            const f2x s6 = f2_mul(f2_mul(s2, s2), s2);
            const f2x t6 = f2_mul(eps4, s6);
            const f2x elj = f2_fma(t6, s6, f2_sub(0ull, t6));
            const f2x ec = f2_add(f2_fma(f2_splat(krf), r2s, invr), f2_splat(-crf));
            e = f2_mul(f2_fma(qq, ec, elj), w);
            // -(dE/dr)/r: LJ (12 t6 s6 - 6 t6) / r^2, Coulomb qq (1/r^3 - 2 krf)
            const f2x flj = f2_mul(t6, f2_fma(s6, f2_splat(12.0f), f2_splat(-6.0f)));
            const f2x fc = f2_mul(qq, f2_fma(invr, invr2, f2_splat(-2.0f * krf)));
            fr = f2_mul(f2_fma(flj, invr2, fc), w);
        }
        eacc = f2_add(eacc, e);
        fix = f2_fma(fr, dx, fix);
        fiy = f2_fma(fr, dy, fiy);
        fiz = f2_fma(fr, dz, fiz);
        fjx = __shfl_sync(FULL_MASK, f2_fma(fr, dx, fjx), src);
        fjy = __shfl_sync(FULL_MASK, f2_fma(fr, dy, fjy), src);
        fjz = __shfl_sync(FULL_MASK, f2_fma(fr, dz, fjz), src);
    }
    // the other group of this half holds the same entry: add its sums, keep this lane's slot
    fjx = f2_add(fjx, __shfl_xor_sync(FULL_MASK, fjx, 8));
    fjy = f2_add(fjy, __shfl_xor_sync(FULL_MASK, fjy, 8));
    fjz = f2_add(fjz, __shfl_xor_sync(FULL_MASK, fjz, 8));
    const bool upper = lane & 8;
    fj.x = upper ? f2_hi(fjx) : f2_lo(fjx);
    fj.y = upper ? f2_hi(fjy) : f2_lo(fjy);
    fj.z = upper ? f2_hi(fjz) : f2_lo(fjz);
    fi.x = -(f2_lo(fix) + f2_hi(fix));
    fi.y = -(f2_lo(fiy) + f2_hi(fiy));
    fi.z = -(f2_lo(fiz) + f2_hi(fiz));
    e32 = f2_lo(eacc) + f2_hi(eacc);
}

// Difference tiles with the adjoint: besides energy and forces, the derivatives
// of the pair energy with respect to each partner's scaled charge, sigma and
// epsilon (LJ: dphi/dsigma_i = eps4 (6 s^12 - 3 s^6) / sigma_ij,
// dphi/deps_i = phi_LJ / (2 eps_i)); j-side sums travel with their slot.
template <int METHOD, bool PBC>
__device__ __forceinline__ void tile_steps_adj(const float4* __restrict__ sp, const float2* __restrict__ sl, float4 pi,
                                               float2 li, unsigned mask, int lane, const ImgBox& B, float rc2,
                                               float alpha, float krf, float crf, float3& fi, float3& fj,
                                               float2& ec, float3& ai, float3& aj) {
    const int src = (lane & kHalf) | ((lane + 1) & (kHalf - 1));  // next lane of this half
    const float inv_ei = li.y > 0.f ? 2.0f / (li.y * li.y) : 0.f;
#pragma unroll 2
    for (int k = 0; k < kHalf; k++) {
        const float4 pj = sp[k];
        const float2 lj = sl[k];
        float dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
        if (PBC) min_image_b(dx, dy, dz, B);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const bool inc = ((mask >> k) & 1u) && r2 < rc2;
        const float r2s = inc ? r2 : 1.0f;
        const float invr = rsqrt_ftz(r2s), invr2 = invr * invr;
        const float sig = li.x + lj.x;
        const float s2 = sig * sig * invr2, s6 = s2 * s2 * s2;
        const float t6 = (li.y * lj.y) * s6;
        const float elj = t6 * s6 - t6;
        const float dsg = sig > 0.f ? (6.0f * t6 * s6 - 3.0f * t6) / sig : 0.f;
        float fr = (12.0f * t6 * s6 - 6.0f * t6) * invr2;
        float gq;
        if (METHOD == 4) {
            const float ar = alpha * r2s * invr;
            const float ex = ex2_ftz(r2s * (-alpha * alpha * kLog2e));
            gq = erfc_as(ar, ex) * invr;
            fr += pi.w * pj.w * (gq + 1.1283791670955126f * alpha * ex) * invr2;
        } else {
            gq = invr + krf * r2s - crf;
            fr += pi.w * pj.w * (invr * invr2 - 2.0f * krf);
        }
        const float on = inc ? 1.0f : 0.0f;
        two_sum_add(ec.x, ec.y, on * (elj + pi.w * pj.w * gq));
        fr *= on;
        const float inv_ej = lj.y > 0.f ? 2.0f / (lj.y * lj.y) : 0.f;
        ai.x += on * gq * pj.w;
        ai.y += on * dsg;
        ai.z += on * elj * inv_ei;
        const float fx = fr * dx, fy = fr * dy, fz = fr * dz;
        fi.x -= fx;
        fi.y -= fy;
        fi.z -= fz;
        fj.x = __shfl_sync(FULL_MASK, fj.x + fx, src);
        fj.y = __shfl_sync(FULL_MASK, fj.y + fy, src);
        fj.z = __shfl_sync(FULL_MASK, fj.z + fz, src);
        aj.x = __shfl_sync(FULL_MASK, aj.x + on * gq * pi.w, src);
        aj.y = __shfl_sync(FULL_MASK, aj.y + on * dsg, src);
        aj.z = __shfl_sync(FULL_MASK, aj.z + on * elj * inv_ej, src);
    }
}

// A warp's shared-memory areas for the pair tiles: the j data of its two half
// tiles, either doubled (64 float4 positions + 64 float2 LJ pairs) or in the
// packed layout (2 x 16 entries of 3 float4), 96 float4 either way; the next
// pass's tile entries (one per half) and j slots, copied asynchronously while the
// current pass runs (no registers held across its pair loop); and each lane's
// bookkeeping for the force and energy output after the loop: (i, j or -1,
// energy slot, kind | flags).
struct TileWarpSmem {
    float4* buf;
    int4* next_t;
    int* next_j;
    int4* meta;
};

// The pairs of tiles [cur, cur_end) (pair pq: tiles 2 pq and 2 pq + 1, one per
// half of the warp; both of one row, since every row holds an even number).
template <int METHOD>
__device__ __forceinline__ void tile_pairs(const Args& a, int cur, int cur_end, const TileWarpSmem& S) {
    const int lane = threadIdx.x & 31;
    const int hf = lane >> 4, l = lane & (kHalf - 1);  // half of the warp, lane within it
    const float rc2 = a.rc2, alpha = a.alpha, krf = a.krf, crf = a.crf;
    // the tile entry and the j slot of the next pass are copied before this
    // pass's pair loop, so that their latency is hidden behind it
    if (l == 0) cp_async16(&S.next_t[hf], a.tiles + 2 * cur + hf);
    cp_async4(&S.next_j[lane], a.tile_j + (size_t)(2 * cur + hf) * kHalf + l);
    for (int pq = cur; pq < cur_end; pq++) {
        const int t = 2 * pq + hf;
        cp_async_wait_all();
        __syncwarp();
        const int4 T = S.next_t[hf];
        const int jraw = S.next_j[lane];
        __syncwarp();
        if (pq + 1 < cur_end) {
            if (l == 0) cp_async16(&S.next_t[hf], a.tiles + t + 2);
            cp_async4(&S.next_j[lane], a.tile_j + (size_t)(t + 2) * kHalf + l);
        }
        const int I16 = T.x, I = I16 >> 1;
        const unsigned z = (unsigned)T.z, wd = (unsigned)T.w;
        const int row = z & 0x0fffffffu, kind = (z >> 28) & 3u;
        const bool atom_tile = (z >> 30) & 1u;
        const int aux = wd & 0xfffffu, slot = (wd >> 20) & 0x7ffu;
        const bool pbc = wd >> 31;
        const RepDev& R = a.reps[a.block_rep[I]];
        const bool diff = kind >= ROW_DIFF1, g2 = kind == ROW_DIFF2;
        const float4* P = kind == ROW_STATE2 ? a.posq2 : a.posq;
        const int i = I16 * kHalf + l;
        float4 pi = P[i];
        const float2 li = a.lj[i];
        int j;
        unsigned mask;
        bool jvalid = true;
        if (atom_tile) {
            jvalid = l < aux;
            j = jvalid ? jraw : i;
            const unsigned vb = aux >= kHalf ? 0xffffu : ((1u << aux) - 1u);
            mask = ((vb >> l) | (vb << (kHalf - l))) & 0xffffu;  // bit k: j-slot (l+k)&15 is a real atom
        } else {
            j = T.y * kHalf + l;
            mask = a.masks[(size_t)(aux - 1) * kHalf + l];
        }
        float4 pj = P[j];
        const float2 lj = a.lj[j];
        if (g2) {
            const float4 di = a.displ[i], dj = a.displ[j];
            pi.x += di.x;
            pi.y += di.y;
            pi.z += di.z;
            pj.x += dj.x;
            pj.y += dj.y;
            pj.z += dj.z;
        }
        if (!pbc) {
            // the image of j nearest block I's centre is the minimum image for every i of the block
            float4 c, h;
            row_box(a, I, kind, c, h);
            float jx = pj.x - c.x, jy = pj.y - c.y, jz = pj.z - c.z;
            float ix = pi.x - c.x, iy = pi.y - c.y, iz = pi.z - c.z;
            min_image3(jx, jy, jz, R);
            min_image3(ix, iy, iz, R);
            pj.x = c.x + jx;
            pj.y = c.y + jy;
            pj.z = c.z + jz;
            pi.x = c.x + ix;
            pi.y = c.y + iy;
            pi.z = c.z + iz;
        }
        // atom tiles without per-pair minimum images need no mask: padding j slots
        // are parked far beyond the cutoff.  The variant is the warp's: masked or
        // per-pair images when either half needs it (the same pairs and arithmetic
        // for the other half).  Both halves are of one row, so of one kind.
        const bool masked_h = !atom_tile || pbc;
        if (!masked_h && !jvalid) pj.x = pj.y = pj.z = 1.0e15f;
        const bool masked = __any_sync(FULL_MASK, masked_h);
        const bool pbc_w = __any_sync(FULL_MASK, pbc);
        // state rows without per-pair images (both halves) run two pairs per
        // instruction on the packed layout, masked or not
        const bool packed = !diff && !pbc_w;
        float4* s_p = S.buf;
        float2* s_l = reinterpret_cast<float2*>(S.buf + 64);
        if (packed) {
            store_packed_j<METHOD>(S.buf + 48 * hf, l, pj, lj);
        } else {
            s_p[32 * hf + l] = pj;
            s_p[32 * hf + l + kHalf] = pj;
            s_l[32 * hf + l] = lj;
            s_l[32 * hf + l + kHalf] = lj;
        }
        __syncwarp();
        const float4* spl = s_p + 32 * hf + l;
        const float2* sll = s_l + 32 * hf + l;
        float3 fi = make_float3(0.f, 0.f, 0.f), fj = make_float3(0.f, 0.f, 0.f);
        float3 ai = make_float3(0.f, 0.f, 0.f), aj = make_float3(0.f, 0.f, 0.f);
        float e32 = 0.f;
        float2 ec = make_float2(0.f, 0.f);  // difference tiles: compensated sum
        const bool adj = diff && a.adjoint;
        {
            const bool diag0 = !atom_tile && T.y == I16;
            const bool skip = atom_tile && aux == 0;  // an empty tile, the filler of an odd row
            S.meta[lane] = make_int4(i, (diag0 || !jvalid) ? -1 : j, row * a.row_cap + slot,
                                        kind | (skip ? 4 : 0) | (adj ? 8 : 0) | (diag0 ? 16 : 0));
        }
        if (packed && masked) {
            // the lane's mask (bit k: slot (l + k) & 15) rotated to slot order (bit s: slot s)
            const unsigned sm = ((mask << l) | (mask >> (kHalf - l))) & 0xffffu;
            tile_steps_x2<METHOD, true>(S.buf + 48 * hf, pi, li, lane, sm, rc2, alpha, krf, crf, fi, fj, e32);
        } else if (packed) {
            tile_steps_x2<METHOD, false>(S.buf + 48 * hf, pi, li, lane, 0u, rc2, alpha, krf, crf, fi, fj, e32);
        } else if (adj) {
            if (pbc_w)
                tile_steps_adj<METHOD, true>(spl, sll, pi, li, mask, lane, img_box(R), rc2, alpha, krf,
                                             crf, fi, fj, ec, ai, aj);
            else
                tile_steps_adj<METHOD, false>(spl, sll, pi, li, mask, lane, img_box(R), rc2, alpha, krf,
                                              crf, fi, fj, ec, ai, aj);
        } else if (diff) {
            if (pbc_w)
                tile_steps<METHOD, true, true, true>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                     alpha, krf, crf, fi, fj, e32, ec);
            else if (masked)
                tile_steps<METHOD, false, true, true>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                      alpha, krf, crf, fi, fj, e32, ec);
            else
                tile_steps<METHOD, false, true, false>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                       alpha, krf, crf, fi, fj, e32, ec);
        } else {
            if (pbc_w)
                tile_steps<METHOD, true, false, true>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                      alpha, krf, crf, fi, fj, e32, ec);
            else if (masked)
                tile_steps<METHOD, false, false, true>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                       alpha, krf, crf, fi, fj, e32, ec);
            else
                tile_steps<METHOD, false, false, false>(spl, sll, pi, li, mask, lane, img_box(R), rc2,
                                                        alpha, krf, crf, fi, fj, e32, ec);
        }
        __syncwarp();
        // the lane's bookkeeping, kept in shared memory across the pair loop
        const int4 m = S.meta[lane];
        const int mi = m.x, mj = m.y, mkind = m.w & 3;
        const bool mdiff = mkind >= ROW_DIFF1, mskip = m.w & 4, madj = m.w & 8, mdiag = m.w & 16;
        // tile energy over the half, in a fixed order: compensated FP32 (TwoSum) on
        // the difference tiles (their sum is u), stored as the (hi, lo) pair that the
        // FP64 row sums add; plain FP32 on the state tiles.  No FP64 instruction
        // runs in this kernel (FP64 is 1/64 of the FP32 rate on this part).  In the two-state mode the state-1 and
        // state-2 tiles of atoms that do not move are the same tiles with the same
        // bits (their j lists differ only in the moving atoms, which come last), so
        // their FP32 sums cancel exactly in u = E2 - E1, which the FP64 row and
        // replica sums carry.
        const float sign = mkind == ROW_DIFF1 ? -1.0f : 1.0f;
        if (mdiff) {
            float es = ec.x, ce = ec.y;
#pragma unroll
            for (int o = kHalf / 2; o > 0; o >>= 1) {
                const float s2 = __shfl_xor_sync(FULL_MASK, es, o), c2 = __shfl_xor_sync(FULL_MASK, ce, o);
                const float t2 = es + s2, bp = t2 - es;
                ce = (ce + c2) + ((es - (t2 - bp)) + (s2 - bp));
                es = t2;
            }
            if (l == 0) a.e_tile[m.z] = make_float2(sign * es, sign * ce);  // exact: sign is +-1
        } else {
            float es = mdiag ? 0.5f * e32 : e32;
#pragma unroll
            for (int o = kHalf / 2; o > 0; o >>= 1) es += __shfl_xor_sync(FULL_MASK, es, o);
            if (l == 0) a.e_tile[m.z] = make_float2(es, 0.f);
        }
        if (!mskip) {
            unsigned long long* Fp = a.F + (mkind == ROW_STATE1 ? 0 : 3 * (size_t)a.NA);
            fix_add_t(Fp + mi, sign * fi.x);
            fix_add_t(Fp + a.NA + mi, sign * fi.y);
            fix_add_t(Fp + 2 * (size_t)a.NA + mi, sign * fi.z);
            if (mj >= 0) {
                fix_add_t(Fp + mj, sign * fj.x);
                fix_add_t(Fp + a.NA + mj, sign * fj.y);
                fix_add_t(Fp + 2 * (size_t)a.NA + mj, sign * fj.z);
            }
            if (madj) {
                unsigned long long* D = a.D;
                fix_add_t(D + mi, sign * ai.x);
                fix_add_t(D + a.NA + mi, sign * ai.y);
                fix_add_t(D + 2 * (size_t)a.NA + mi, sign * ai.z);
                if (mj >= 0) {
                    fix_add_t(D + mj, sign * aj.x);
                    fix_add_t(D + a.NA + mj, sign * aj.y);
                    fix_add_t(D + 2 * (size_t)a.NA + mj, sign * aj.z);
                }
            }
        }
    }
}

// MINB: CTAs per SM the registers are budgeted for: 4 (64 registers, some spills
// around the pair loop) or 3 (80 registers, none); the autotuner's CTAs per SM
// pick the variant.
template <int METHOD, bool DYN, int MINB>
__global__ void __launch_bounds__(kTileThreads, MINB) k_tiles(Args a) {
    __shared__ float4 s_buf[kTileThreads / 32][96];
    __shared__ int4 s_next_t[kTileThreads / 32][2];
    __shared__ int s_next_j[kTileThreads / 32][32];
    __shared__ int4 s_meta[kTileThreads / 32][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const TileWarpSmem S{s_buf[w], s_next_t[w], s_next_j[w], s_meta[w]};
    int ntiles = a.status->tile_count;
    if (ntiles > a.tile_cap) ntiles = a.tile_cap;
    const int npairs = ntiles >> 1;  // every row holds an even number of tiles
    // A warp takes two consecutive tiles (one per half; the same row).  Large
    // lists: pairs handed out kTileGrab at a time from a counter (the next grab
    // requested before the current pairs are processed), so that warps finish
    // together.  Small lists (a few pairs per warp): warp w takes pairs w, w + nw, ...
    // (DYN, chosen by the host from the size of the row list)
    int mine = 0;
    if (DYN && lane == 0) mine = atomicAdd(&a.status->next_tile, kTileGrab);
    int cur = DYN ? __shfl_sync(FULL_MASK, mine, 0) : ((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    while (cur < npairs) {
        if (DYN && lane == 0) mine = atomicAdd(&a.status->next_tile, kTileGrab);
        const int cur_end = DYN ? min(cur + kTileGrab, npairs) : cur + 1;
        tile_pairs<METHOD>(a, cur, cur_end, S);
        cur = DYN ? __shfl_sync(FULL_MASK, mine, 0) : cur + ((gridDim.x * blockDim.x) >> 5);
    }
}

// Lists and pair tiles in one persistent kernel: a warp takes a row (longest
// first, as k_find), builds its tiles when this evaluation builds the lists, and
// evaluates them at once, while they are in L1 / L2; with kept lists (a skin) it
// evaluates the row's tiles of the last build.  The finder's load-latency-bound
// phases of some warps run beside the issue-bound pair loops of others on the
// same SM.  Five CTAs of four warps per SM (102 registers, 45 KB of shared memory
// each).
constexpr int kFusedMinBlocks = 5;

template <int METHOD, bool TRIC>
__global__ void __launch_bounds__(kFindWarps * 32, kFusedMinBlocks) k_find_tiles(Args a) {
    __shared__ int s_stage[kFindWarps][kStageAtoms];
    __shared__ float4 s_ipos[kFindWarps][32];
    __shared__ float4 s_buf[kFindWarps][96];
    __shared__ int4 s_next_t[kFindWarps][2];
    __shared__ int s_next_j[kFindWarps][32];
    __shared__ int4 s_meta[kFindWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const TileWarpSmem S{s_buf[w], s_next_t[w], s_next_j[w], s_meta[w]};
    const bool build = a.status->rebuild != 0;
    if (build && a.skin_half2 > 0.f)  // the positions of this build, for the displacement test
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.NA; s += gridDim.x * blockDim.x)
            a.posq_ref[s] = a.posq[s];
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int mine = a.nrows;
    while (k < a.nrows) {
        if (lane == 0) mine = nw < a.nrows ? nw + atomicAdd(&a.status->next_row, 1) : a.nrows;
        const int row = a.nrows - 1 - k;
        if (build) find_row<TRIC>(a, row, lane, s_stage[w], s_ipos[w]);
        __syncwarp();
        // the row's tiles (written by this warp just now, or by an earlier build)
        const int n = a.row_count[row], tb = a.row_tbase[row];
        if (n > 0 && tb + n <= a.tile_cap) tile_pairs<METHOD>(a, tb >> 1, (tb + n) >> 1, S);
        k = __shfl_sync(FULL_MASK, mine, 0);
    }
}

void launch_find_tiles(const Args& a, cudaStream_t s) {
    static int per_sm = 0, sms = 0;
    if (per_sm == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int p4 = 0, p2 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p4, k_find_tiles<4, true>, kFindWarps * 32, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p2, k_find_tiles<2, true>, kFindWarps * 32, 0);
        per_sm = std::max(1, std::min(p4, p2));
    }
    const int blocks = std::min(per_sm * sms, (a.nrows + kFindWarps - 1) / kFindWarps);
    if (a.method == 4) {
        if (a.any_tric)
            k_find_tiles<4, true><<<blocks, kFindWarps * 32, 0, s>>>(a);
        else
            k_find_tiles<4, false><<<blocks, kFindWarps * 32, 0, s>>>(a);
    } else {
        if (a.any_tric)
            k_find_tiles<2, true><<<blocks, kFindWarps * 32, 0, s>>>(a);
        else
            k_find_tiles<2, false><<<blocks, kFindWarps * 32, 0, s>>>(a);
    }
}

int tiles_kernel_blocks_per_sm() {
    int n4 = 0, n2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n4, k_tiles<4, true, 4>, kTileThreads, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n2, k_tiles<2, true, 4>, kTileThreads, 0);
    return n4 < n2 ? n4 : n2;
}

template <int METHOD, bool DYN>
static void launch_tiles_m(const Args& a, int grid, cudaStream_t s) {
    if (a.tile_wide)
        k_tiles<METHOD, DYN, 3><<<grid, kTileThreads, 0, s>>>(a);
    else
        k_tiles<METHOD, DYN, 4><<<grid, kTileThreads, 0, s>>>(a);
}

void launch_tiles(const Args& a, int grid, cudaStream_t s) {
    if (a.method == 4) {
        if (a.tile_dynamic)
            launch_tiles_m<4, true>(a, grid, s);
        else
            launch_tiles_m<4, false>(a, grid, s);
    } else {
        if (a.tile_dynamic)
            launch_tiles_m<2, true>(a, grid, s);
        else
            launch_tiles_m<2, false>(a, grid, s);
    }
}

}  // namespace atm
