// Reaction-field nonbonded energy and forces for callers that cannot allocate
// device memory.
//
// Some callers of this library run where cudaMalloc is not an option: code
// that owns all device memory through its own pool or arena, code running
// while another component forbids new allocations (a memory budget already
// handed out, an allocator that must not be re-entered), or host code that
// simply must not add allocation latency to its step.  They get this one entry
// point, which takes every input and output from the caller and keeps its
// scratch (64-bit fixed-point force accumulators and per-CTA energy partials)
// in a file-scope __device__ array that every GPU loading the library holds
// until the process exits.
//
// It is the all-pairs variant of the pair-tile kernel of kernels.cu for
// CutoffPeriodic (reaction field) with exclusions, for at most
// kNoAllocMaxAtoms particles.  The rest of the library is untouched by it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/atm_capi.h"
#include "model.h"

namespace atm {
namespace {

constexpr int kNoAllocMaxAtoms = 16384;  // particles per call
constexpr int kNoAllocCtas = 512;        // CTAs of the tile pass (one energy partial each)
constexpr int kNoAllocThreads = 256;
constexpr int kMaxDevices = 64;
constexpr double kFix = 4294967296.0;  // 2^32 fixed-point units per kJ/mol/nm

struct NoAllocScratch {
    unsigned long long force[3 * kNoAllocMaxAtoms];
    double energy[kNoAllocCtas];
};

// The scratch every call shares (about 400 KB per GPU).
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_setup_mutex;
NoAllocScratch* g_scratch_ptr[kMaxDevices] = {nullptr};

__global__ void k_noalloc_clear(NoAllocScratch* s, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < 3 * n) s->force[k] = 0ull;
    if (k < kNoAllocCtas) s->energy[k] = 0.0;
}

__device__ __forceinline__ void tri_index(long long t, int nb, int& I, int& J) {
    // tile t of the upper triangle (I <= J) of an nb x nb block grid, row-major
    long long lo = 0, hi = nb - 1;
    while (lo < hi) {  // largest I with first(I) <= t, first(I) = I*nb - I*(I-1)/2
        long long mid = (lo + hi + 1) >> 1;
        long long first = mid * nb - mid * (mid - 1) / 2;
        if (first <= t) lo = mid;
        else hi = mid - 1;
    }
    I = (int)lo;
    long long first = lo * nb - lo * (lo - 1) / 2;
    J = (int)(lo + (t - first));
}

__global__ void __launch_bounds__(kNoAllocThreads) k_noalloc_tiles(
    NoAllocScratch* s, int n, const double* __restrict__ pos, const double* __restrict__ q,
    const double* __restrict__ sig, const double* __restrict__ eps, const int* __restrict__ ex_start,
    const int* __restrict__ ex_list, double Lx, double Ly, double Lz, float rc2, float krf, float crf) {
    __shared__ double red[kNoAllocThreads / 32];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int nb = (n + 31) / 32;
    const long long ntiles = (long long)nb * (nb + 1) / 2;
    const float fLx = (float)Lx, fLy = (float)Ly, fLz = (float)Lz;
    const float iLx = 1.0f / fLx, iLy = 1.0f / fLy, iLz = 1.0f / fLz;
    const float sqk = 11.787089759563214f;  // sqrt(138.935456)
    double ewarp = 0.0;
    for (long long t = gw; t < ntiles; t += nw) {
        int I, J;
        tri_index(t, nb, I, J);
        const int i = I * 32 + lane;
        const int j0 = J * 32 + lane;
        const bool vi = i < n;
        float xi = 0.f, yi = 0.f, zi = 0.f, qi = 0.f, si = 0.f, ei = 0.f;
        int e0 = 0, e1 = 0;
        if (vi) {
            xi = (float)(pos[3 * i] - Lx * floor(pos[3 * i] / Lx));
            yi = (float)(pos[3 * i + 1] - Ly * floor(pos[3 * i + 1] / Ly));
            zi = (float)(pos[3 * i + 2] - Lz * floor(pos[3 * i + 2] / Lz));
            qi = (float)q[i] * sqk;
            si = 0.5f * (float)sig[i];
            ei = 2.0f * sqrtf((float)eps[i]);
            e0 = ex_start[i];
            e1 = ex_start[i + 1];
        }
        float xj = 0.f, yj = 0.f, zj = 0.f, qj = 0.f, sj = 0.f, ej = 0.f;
        if (j0 < n) {
            xj = (float)(pos[3 * j0] - Lx * floor(pos[3 * j0] / Lx));
            yj = (float)(pos[3 * j0 + 1] - Ly * floor(pos[3 * j0 + 1] / Ly));
            zj = (float)(pos[3 * j0 + 2] - Lz * floor(pos[3 * j0 + 2] / Lz));
            qj = (float)q[j0] * sqk;
            sj = 0.5f * (float)sig[j0];
            ej = 2.0f * sqrtf((float)eps[j0]);
        }
        const bool diag = (I == J);
        float fix = 0.f, fiy = 0.f, fiz = 0.f, fjx = 0.f, fjy = 0.f, fjz = 0.f;
        double e = 0.0;
        const int src = (lane + 1) & 31;
        for (int k = 0; k < 32; k++) {
            const int j = J * 32 + ((lane + k) & 31);
            bool ok = vi && j < n && !(diag && k == 0);
            float dx = xj - xi, dy = yj - yi, dz = zj - zi;
            dx -= fLx * rintf(dx * iLx);
            dy -= fLy * rintf(dy * iLy);
            dz -= fLz * rintf(dz * iLz);
            float r2 = dx * dx + dy * dy + dz * dz;
            ok = ok && r2 < rc2;
            if (ok) {
                for (int m = e0; m < e1; m++)
                    if (ex_list[m] == j) ok = false;
            }
            if (ok) {
                float invr = rsqrtf(r2), invr2 = invr * invr;
                float sg = si + sj;
                float s2 = sg * sg * invr2, s6 = s2 * s2 * s2;
                float ep = ei * ej;
                float qq = qi * qj;
                float en = ep * (s6 * s6 - s6) + qq * (invr + krf * r2 - crf);
                float fr = ep * (12.0f * s6 * s6 - 6.0f * s6) * invr2 + qq * (invr * invr2 - 2.0f * krf);
                e += (double)en;
                fix -= fr * dx;
                fiy -= fr * dy;
                fiz -= fr * dz;
                fjx += fr * dx;
                fjy += fr * dy;
                fjz += fr * dz;
            }
            xj = __shfl_sync(0xffffffffu, xj, src);
            yj = __shfl_sync(0xffffffffu, yj, src);
            zj = __shfl_sync(0xffffffffu, zj, src);
            qj = __shfl_sync(0xffffffffu, qj, src);
            sj = __shfl_sync(0xffffffffu, sj, src);
            ej = __shfl_sync(0xffffffffu, ej, src);
            fjx = __shfl_sync(0xffffffffu, fjx, src);
            fjy = __shfl_sync(0xffffffffu, fjy, src);
            fjz = __shfl_sync(0xffffffffu, fjz, src);
        }
        ewarp += diag ? 0.5 * e : e;
        if (vi) {
            atomicAdd(&s->force[i], (unsigned long long)__float2ll_rn(fix * 4294967296.0f));
            atomicAdd(&s->force[n + i], (unsigned long long)__float2ll_rn(fiy * 4294967296.0f));
            atomicAdd(&s->force[2 * n + i], (unsigned long long)__float2ll_rn(fiz * 4294967296.0f));
        }
        if (!diag && j0 < n) {
            atomicAdd(&s->force[j0], (unsigned long long)__float2ll_rn(fjx * 4294967296.0f));
            atomicAdd(&s->force[n + j0], (unsigned long long)__float2ll_rn(fjy * 4294967296.0f));
            atomicAdd(&s->force[2 * n + j0], (unsigned long long)__float2ll_rn(fjz * 4294967296.0f));
        }
    }
    for (int o = 16; o > 0; o >>= 1) ewarp += __shfl_xor_sync(0xffffffffu, ewarp, o);
    if (lane == 0) red[warp] = ewarp;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; w++) sum += red[w];
        s->energy[blockIdx.x] = sum;  // one slot per CTA: no order dependence
    }
}

__global__ void k_noalloc_finish(const NoAllocScratch* s, int n, double* energy, double* forces) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        for (int a = 0; a < 3; a++)
            forces[3 * k + a] = (double)(long long)s->force[a * n + k] * (1.0 / kFix);
    }
    if (k == 0) {
        double sum = 0.0;
        for (int c = 0; c < kNoAllocCtas; c++) sum += s->energy[c];
        *energy = sum;
    }
}

// Device address of the scratch on the current device, looked up once per
// device (cudaGetSymbolAddress with that device current).
NoAllocScratch* scratch_for_current_device() {
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) throw Error(ATM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(err));
    if (dev < 0 || dev >= kMaxDevices) throw Error(ATM_ERR_UNSUPPORTED, "device ordinal too large");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess)
            throw Error(ATM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(err));
        g_scratch_ptr[dev] = (NoAllocScratch*)p;
    }
    return g_scratch_ptr[dev];
}

}  // namespace

// Records the message returned by atm_last_error() (defined with the other entry points).
void set_last_error(const std::string& msg);

}  // namespace atm

extern "C" int atm_rf_nonbonded_noalloc(int n, const double* d_pos, const double* d_charge, const double* d_sigma,
                                        const double* d_epsilon, const int* d_excl_start, const int* d_excl,
                                        const double* box, double cutoff, double eps_rf, double* d_energy,
                                        double* d_forces, void* stream) {
    using namespace atm;
    try {
        if (n <= 0 || !d_pos || !d_charge || !d_sigma || !d_epsilon || !d_excl_start || !d_excl || !box ||
            !d_energy || !d_forces)
            throw Error(ATM_ERR_INVALID_ARGUMENT, "null pointer or empty system");
        if (n > kNoAllocMaxAtoms)
            throw Error(ATM_ERR_INVALID_ARGUMENT,
                        "atm_rf_nonbonded_noalloc: " + std::to_string(n) + " particles exceed the maximum of " +
                            std::to_string(kNoAllocMaxAtoms));
        if (!(cutoff > 0) || !(eps_rf > 0)) throw Error(ATM_ERR_INVALID_ARGUMENT, "bad cutoff or dielectric");
        for (int a = 0; a < 3; a++)
            if (!(box[a] >= 2.0 * cutoff))
                throw Error(ATM_ERR_INVALID_ARGUMENT, "the box must be at least twice the cutoff");
        NoAllocScratch* s = scratch_for_current_device();
        cudaStream_t st = (cudaStream_t)stream;
        double krf = (eps_rf - 1.0) / ((2.0 * eps_rf + 1.0) * cutoff * cutoff * cutoff);
        double crf = 3.0 * eps_rf / ((2.0 * eps_rf + 1.0) * cutoff);
        int clear_blocks = (3 * n + kNoAllocThreads - 1) / kNoAllocThreads;
        if (clear_blocks * kNoAllocThreads < kNoAllocCtas) clear_blocks = kNoAllocCtas / kNoAllocThreads;
        k_noalloc_clear<<<clear_blocks, kNoAllocThreads, 0, st>>>(s, n);
        k_noalloc_tiles<<<kNoAllocCtas, kNoAllocThreads, 0, st>>>(s, n, d_pos, d_charge, d_sigma, d_epsilon,
                                                                  d_excl_start, d_excl, box[0], box[1], box[2],
                                                                  (float)(cutoff * cutoff), (float)krf, (float)crf);
        k_noalloc_finish<<<(n + kNoAllocThreads - 1) / kNoAllocThreads, kNoAllocThreads, 0, st>>>(s, n, d_energy,
                                                                                                    d_forces);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) throw Error(ATM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(err));
        set_last_error("");
        return ATM_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    }
}
