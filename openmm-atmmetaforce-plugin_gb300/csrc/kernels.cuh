// Device data layout and kernel interfaces of the ATM evaluation engine.
//
// Atoms of all replicas live in one "slot" space: each replica's atoms are
// reordered (non-moving molecules along a Hilbert curve, then each displacement
// class) and padded so that every 32-slot block belongs to one replica and one
// displacement class.  Forces accumulate as 64-bit fixed point (2^32 units per
// kJ/mol/nm) so that sums are exact and independent of launch order; energies
// are summed in FP64 through per-tile / per-CTA partials in fixed order.
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace atm {

constexpr int kTile = 32;
constexpr int kHalf = 16;  // pair tiles are half blocks: 16 i atoms x 16 j slots
constexpr double kFixScale = 4294967296.0;  // 2^32
constexpr int kOrder = 5;  // PME B-spline order (OpenMM's)
constexpr float kGridScale = 33554432.0f;  // charge grids: 2^25 int32 fixed-point units per e

// round(v * 2^32) as a 64-bit two's-complement integer, from 32-bit conversions
// only (64-bit conversions issue on the FP64 pipe, which is narrow on this GPU).
// With h = floor(v), f = v - h is exact and lies in [0, 1), so
// round(v 2^32) = h 2^32 + round(f 2^32), and f 2^32 <= 2^32 - 2^8 never rounds up
// to 2^32.  Equal to cvt.rni.s64.f32 of v 2^32 for |v| < 2^31 (both saturate beyond).
#ifdef __CUDACC__
__device__ __forceinline__ unsigned long long fix_bits(float v) {
    const float h = floorf(v);
    const unsigned lo = __float2uint_rn((v - h) * 4294967296.0f);
    const unsigned hi = (unsigned)__float2int_rz(h);
    return ((unsigned long long)hi << 32) | lo;
}

// v 2^-32 as a double (a fixed-point force sum in kJ/mol/nm): one conversion, then
// the exact scaling by 2^-32 as an exponent decrement (|v| >= 1 stays normal).
__device__ __forceinline__ double fix_scaled(long long v) {
    const double d = (double)v;
    return v == 0 ? 0.0 : __longlong_as_double(__double_as_longlong(d) - (32LL << 52));
}
#endif

// The z-row stride (words) of a spreading brick's int32 accumulator: at least n,
// and, when at most 6 words of padding achieve it, such that the 5 x 5 (y, z)
// patch of a stencil that a warp adds with one instruction falls in 25 different
// shared-memory banks (b p + c, b, c < 5, distinct modulo 32); otherwise n.
__host__ __device__ inline int spread_row_stride(int n) {
    for (int p = n; p <= n + 6; p++) {
        unsigned used = 0u;
        bool ok = true;
        for (int b = 0; b < 5 && ok; b++)
            for (int c = 0; c < 5; c++) {
                const unsigned bit = 1u << ((b * p + c) & 31);
                if (used & bit) {
                    ok = false;
                    break;
                }
                used |= bit;
            }
        if (ok) return p;
    }
    return n;
}

// Row kinds of the pair-tile lists.
enum RowKind { ROW_STATE1 = 0, ROW_STATE2 = 1, ROW_DIFF1 = 2, ROW_DIFF2 = 3 };

// Result record layout (matches ATM_RES_* in include/atm_capi.h).
enum Res {
    RES_ENERGY = 0, RES_PERT, RES_SP, RES_W, RES_U, RES_E0, RES_BFP, RES_FP, RES_E1, RES_E2,
    RES_DL1, RES_DL2, RES_DALPHA, RES_DU0, RES_DW0, RES_STATUS, RES_DWDU, NUM_RES
};

// Per-replica constants and offsets (device copy refreshed every evaluation).
// One Stockham stage of a 1D transform of length N: radix R, Ns the product of
// the earlier stages' radices, nb = N / R butterflies, step = N / (Ns R) (the
// twiddle exponent's stride), mNs = ceil(2^32 / Ns) for the division by Ns.
struct FftStage {
    int R, Ns, nb, step;
    unsigned mNs;
    int pad[3];
};

struct RepDev {
    float box[4];      // L (x,y,z), unused
    float ibox[4];     // 1/L
    double boxd[3];
    double iboxd[3];          // 1/L in FP64 (FP64 division is slow on this part)
    int slot_begin, slot_end;
    int block_begin, block_end;
    int mov_block_begin;      // first moving block (== block_end when none)
    int in_off;               // first atom of this replica in user-order arrays
    int n;                    // atoms (user order)
    int K[3];                 // PME grid
    int mod_off[3];           // offsets of the B-spline moduli (per dimension)
    long long real_off;       // first float of this replica's two real grids
    long long cplx_off;       // first complex of its two spectra
    int nbrick[3];            // spreading bricks per dimension
    int bsz[3];               // brick size (grid points) per dimension
    int brick_cta_b;          // first spreading CTA of this replica (2 x bricks CTAs)
    int row1_b, row1_e;       // rows of state 1 (full and difference modes)
    int row2_b, row2_e;       // rows of state 2 (full) or of the difference tiles (diff)
    int exc_cta_b, exc_cta_e; // exception-kernel CTAs (energy partials)
    int conv_cta_b, conv_cta_e;
    int var_nb;               // the NonbondedForce is in the ATM variable groups
    int tw_off[3];            // FFT twiddle tables of the three grid dimensions
    int fft_plan[3];          // FFT stage plans per dimension: first stage | stage count << 24
    int pad0[1];
    double e_self;            // PME self energy (FP64, host)
    double e_disp;            // dispersion correction (FP64, host)
    double params[9];         // ATM globals
    // Triclinic boxes, OpenMM's reduced form: a = (box[0], 0, 0),
    // b = (tilt[0], box[1], 0), c = (tilt[1], tilt[2], box[2])
    double tiltd[4];          // b_x, c_x, c_y (FP64), 0
    float tilt[4];            // the same in FP32
    float recip[8];           // reciprocal box rows r00, r10, r11, r20, r21, r22 (fractional coordinates)
    int tric;                 // 1: some tilt is nonzero
    float wmin;               // smallest distance between opposite faces of the box (nm)
    int pad1[2];
};

#ifdef __CUDACC__
// OpenMM's minimum image in a reduced box: subtract c, then b, then a, each
// rounded to the nearest multiple (per axis when the box is orthorhombic; the
// identity without periodic boundaries, where the inverse box is 0).
__device__ __forceinline__ void min_image3(float& x, float& y, float& z, const RepDev& R) {
    if (R.tric) {
        const float kz = rintf(z * R.ibox[2]);
        x -= kz * R.tilt[1];
        y -= kz * R.tilt[2];
        z -= kz * R.box[2];
        const float ky = rintf(y * R.ibox[1]);
        x -= ky * R.tilt[0];
        y -= ky * R.box[1];
        x -= R.box[0] * rintf(x * R.ibox[0]);
    } else {
        x -= R.box[0] * rintf(x * R.ibox[0]);
        y -= R.box[1] * rintf(y * R.ibox[1]);
        z -= R.box[2] * rintf(z * R.ibox[2]);
    }
}
__device__ __forceinline__ void min_image3d(double& x, double& y, double& z, const RepDev& R) {
    if (R.tric) {
        const double kz = rint(z * R.iboxd[2]);
        x -= kz * R.tiltd[1];
        y -= kz * R.tiltd[2];
        z -= kz * R.boxd[2];
        const double ky = rint(y * R.iboxd[1]);
        x -= ky * R.tiltd[0];
        y -= ky * R.boxd[1];
        x -= R.boxd[0] * rint(x * R.iboxd[0]);
    } else {
        x -= R.boxd[0] * rint(x * R.iboxd[0]);
        y -= R.boxd[1] * rint(y * R.iboxd[1]);
        z -= R.boxd[2] * rint(z * R.iboxd[2]);
    }
}
// The periodic image inside the unit cell (fractional coordinates in [0, 1)).
__device__ __forceinline__ void wrap3(float& x, float& y, float& z, const RepDev& R) {
    const float kz = floorf(z * R.ibox[2]);
    x -= kz * R.tilt[1];
    y -= kz * R.tilt[2];
    z -= kz * R.box[2];
    const float ky = floorf(y * R.ibox[1]);
    x -= ky * R.tilt[0];
    y -= ky * R.box[1];
    x -= R.box[0] * floorf(x * R.ibox[0]);
}
__device__ __forceinline__ void wrap3d(double& x, double& y, double& z, const RepDev& R) {
    const double kz = floor(z * R.iboxd[2]);
    x -= kz * R.tiltd[1];
    y -= kz * R.tiltd[2];
    z -= kz * R.boxd[2];
    const double ky = floor(y * R.iboxd[1]);
    x -= ky * R.tiltd[0];
    y -= ky * R.boxd[1];
    x -= R.boxd[0] * floor(x * R.iboxd[0]);
}
// Fractional coordinates (along a, b, c) of a position: p . column d of the reciprocal box.
__device__ __forceinline__ void frac3(float x, float y, float z, const RepDev& R, float* f) {
    f[0] = fmaf(z, R.recip[3], fmaf(y, R.recip[1], x * R.recip[0]));
    f[1] = fmaf(z, R.recip[4], y * R.recip[2]);
    f[2] = z * R.recip[5];
}
#endif

// Parameters of one exception pair (x: chargeProd * ke, y: sigma, z: epsilon,
// w: ke * q_i * q_j for the Ewald exclusion correction).
struct __align__(16) ExcParam {
    double x, y, z, w;
};

struct Status {
    int tile_count;   // tiles appended by the finder
    int overflow;     // bit 0: tile list, bit 1: row capacity (of the last list build)
    int max_row;      // largest row seen
    int next_tile;    // work counter of the pair-tile kernel (tiles handed out)
    int next_row;     // work counter of the tile finder (rows handed out)
    int rebuild;      // 1: the lists are built in this evaluation
    unsigned disp2;   // largest squared displacement since the last build (float bits)
    int sticky;       // overflow bits of every build since the host last cleared them
};

// Arguments shared by the kernels of one engine (passed by value).
struct Args {
    // sizes
    int R, NA, NB, nrows, row_cap, tile_cap, n_in;
    int full;                 // 1: two full states, 0: state 1 + difference
    // method
    int method;               // 2 reaction field, 4 PME
    float rc2, alpha, krf, crf;
    // neighbour lists: built at the list cutoff rc + skin and kept while no atom
    // has moved more than skin / 2 since the build (skin 0: built every evaluation)
    float rcl2;               // (rc + skin)^2
    float skin_half2;         // (skin / 2)^2
    float4* posq_ref;         // NA: positions at the last build
    const int* list_ctl;      // device control word: [0] = 1 forces a build
    unsigned* rep_hmax;       // R: largest half-extent norm of a block (float bits; triclinic boxes)
    int any_tric;             // 1: some replica's box is triclinic
    long long* list_counts;   // device: evaluations, list builds
    double alphad, cutoffd;
    // replicas
    RepDev* reps;
    // user-order inputs and outputs
    const double* pos_in;     // 3*n_in
    const double* displ_in;   // 3*n_in
    const int* slot_of;       // n_in
    double* f_out;            // 3*n_in (ATM force)
    double* const* io;        // device cells, copied from the host by every evaluation: io[0] the
                              // caller's device positions, read in place of pos_in; io[1] the
                              // caller's force buffer (device, or page-locked host memory
                              // written over the host link) in place of f_out; io[2] the
                              // caller's device result records (a copy of results); null: unused
    double* f_nb;             // 3*n_in (state-1 nonbonded force) or null
    // slot arrays
    const int* orig;          // NA: user index within the replica, -1 for padding
    const float* qs;          // NA: charge * sqrt(1/(4 pi eps0))
    const float2* lj;         // NA: (sigma/2, 2 sqrt(eps))
    const float4* displ;      // NA: displacement (sorted)
    float4* posq;             // NA: wrapped positions + scaled charge (state 1)
    float4* posq2;            // NA: state 2 (full mode) or null
    // blocks
    const int* block_rep;     // NB
    const int* block_cls;     // NB: displacement class (0 = not moving)
    const float4* block_d;    // NB: displacement of the block's class
    int n_mov_blocks;         // blocks of moving atoms (all replicas)
    const int* mov_blocks;
    float4* bb_c;             // NB: bounding-box centres (state 1)
    float4* bb_h;             // NB: half extents
    float4* bb_c2;            // NB: state 2 (full mode)
    float4* bb_h2;
    // rows and tiles
    const int4* row_desc;     // nrows: (I, kind, replica, part | parts << 8)
    int* row_count;           // nrows
    int* row_tbase;           // nrows: first tile of each row in the last build
    const int* ex_start;      // NB+1: exclusion tiles of row I (regular rows)
    const int2* ex_ent;       //   (J, mask id)
    const int* dx_start;      // NB+1: cross-class exclusion tiles (difference rows)
    const int2* dx_ent;
    const int* exs_start;     // NB+1: 16 x 16 sub-tiles of the exclusion tiles of row I
    const int4* exs_ent;      //   (I16, J16, mask16 id, 0)
    const int* dxs_start;     // NB+1: sub-tiles of the cross-class exclusion tiles
    const int4* dxs_ent;
    const uint32_t* masks;    // 16 words per mask (16 x 16 sub-tiles, low 16 bits)
    int4* tiles;              // tile_cap entries, see tiles.cu for the encoding
    int tile_dynamic;         // 1: pair tiles handed out from a counter (large lists)
    int tile_wide;            // 1: the pair-tile variant budgeted for 3 CTAs per SM (80 registers)
    int fused;                // 1: lists and pair tiles in one persistent kernel (k_find_tiles)
    int* tile_j;              // 32 j slots per tile (atom tiles)
    float2* e_tile;           // nrows*row_cap: tile energies as (hi, lo) FP32 pairs, summed in FP64 per row
    int fin_ctas;             // finalize CTAs per replica (row sums), the last one merges
    double* fin_part;         // R x fin_ctas x 2: row-energy partials (state 1, state 2 / difference)
    int* fin_count;           // R: finalize CTAs done (the last resets it to 0)
    Status* status;
    // forces (fixed point), planes of NA: [F1x F1y F1z | F2x F2y F2z]
    unsigned long long* F;
    // adjoint (difference mode): planes of NA of d(U2-U1)/d(q*sqrt(ke)), d/dsigma,
    // d/depsilon, int64 fixed point; null when the adjoint is off
    int adjoint;
    unsigned long long* D;
    double sqrt_ke;
    // exceptions (user-order indices, grouped by replica)
    int n_exc;
    const int4* exc_ij;       // (i_in, j_in, replica, cross)
    const ExcParam* exc_p;    // (chargeProd*ke, sigma, epsilon, q_i q_j ke)
    double* e_part_exc;       // 3 per CTA: state 1, state 2, difference
    int exc_ctas;
    const int* exc_cta_first; // first exception of each CTA
    // PME
    int brick_ctas;           // spreading CTAs (all replicas)
    int brick_smem;           // dynamic shared memory of a spreading CTA (bytes)
    int spread_owner;         // 1: the charge grids are int32, zeroed before the spreading and
                              // summed by integer atomics (the forward transform reads int32):
                              // every atom spread once, by the brick of its stencil base, or
    int spread_atoms;         //   (1) by its own warp straight into the grids (small systems)
    const int* brick_cta_rep; // replica of each spreading CTA
    float* qreal;             // real grids (charge, then potential)
    float2* qcplx;            // spectra
    const float* moduli;      // B-spline moduli, per replica per dimension
    double* e_part_conv;      // 2 per CTA: E_rec1, E_rec2 - E_rec1
    int conv_ctas;
    // library transforms (grids whose planes exceed shared memory): the
    // convolution kernel's CTAs
    const int* conv_cta_rep;  // replica of each conv CTA
    const long long* conv_cta_first;  // first complex element of each conv CTA
    // hand-written transforms (pme_fft.cu)
    int use_fft;              // 1: k_fft_zy / k_fft_x_conv / k_ifft_yz
    const float2* fft_tw;     // twiddles w_N^k = exp(-2 pi i k / N), per replica and dimension
    const FftStage* fft_stages;  // stage plans (RepDev::fft_plan indexes them)
    int fft_plane_ctas;       // (grid, x-plane) CTAs of all replicas
    const int2* fft_plane;    //   (replica, grid * K0 + x)
    int fft_plane_smem;       // dynamic shared memory of a plane CTA (bytes)
    const int4* fft_conv;     // conv CTAs: (replica, ky, kz0, kz1)
    int fft_conv_smem;
    float* influence;         // influence function per replica, [ky][x][kz] at cplx_off / 2
    long long n_real_total;
    // results
    double* results;          // R * NUM_RES
    double* matrix;           // R * R
    const double* beta;       // device scalar
};

void launch_prepare(const Args& a, cudaStream_t s);
void launch_decide(const Args& a, cudaStream_t s);
void launch_find(const Args& a, cudaStream_t s);
void launch_tiles(const Args& a, int grid, cudaStream_t s);
void launch_find_tiles(const Args& a, cudaStream_t s);
void launch_exceptions(const Args& a, cudaStream_t s);
void launch_spread(const Args& a, cudaStream_t s);
void launch_conv(const Args& a, cudaStream_t s);
void launch_gather(const Args& a, cudaStream_t s);
void launch_fft_forward(const Args& a, cudaStream_t s);
void launch_fft_conv(const Args& a, cudaStream_t s);
void launch_fft_inverse(const Args& a, cudaStream_t s);
int fft_plane_smem_bytes(int K1, int K2);
// Stages of a 1D transform of length N appended to out; returns first | count << 24.
int fft_plan_stages(int N, std::vector<FftStage>& out);
void launch_influence(float* G, const float* moduli, const int* mod_off, const int* K, const double* recip,
                      double volume, double alpha, cudaStream_t s);
int fft_conv_smem_bytes(int K0, int nz);
void launch_finalize(const Args& a, cudaStream_t s);
void launch_output(const Args& a, cudaStream_t s);
void launch_matrix(const Args& a, cudaStream_t s);
// Gradients of sum_r g_r W_r (host-provided upstream gradient g, device array of R):
// positions, displacements, charges, sigmas, epsilons (user order, n_in each; x3 for
// vectors) and the 5 softplus parameters per replica (R x 5).  Outputs nullable.
void launch_adjoint(const Args& a, const double* g, double* dx, double* dd, double* dq, double* dsig, double* deps,
                    double* dpar, cudaStream_t s);
int tiles_kernel_blocks_per_sm();
int find_warps_per_sm();
constexpr int kTileThreads = 256;

}  // namespace atm
