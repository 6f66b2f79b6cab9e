// Host side of the GPU evaluation engine: atom layout, buffers, cuFFT plans and
// the CUDA graph that runs one ATM evaluation of all replicas.
//
// Reference correspondence: the engine replaces ATMMetaForceImpl's two linked
// inner contexts (ATMMetaForceImpl.cpp:32-67,94-95) and CommonCalcATMMetaForceKernel
// (CommonATMMetaForceKernels.cpp:78-251): CopyState becomes the displacement of
// the state-2 slots (k_prepare), the two inner evaluations become one pass over
// both states (or over state 1 plus the ligand difference), and execute() runs
// on the device in FP64 with no host round trip for E1/E2.
#include "engine.h"

#include <algorithm>
#include <cstdlib>
#include <fstream>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <set>
#include <thread>
#include <sstream>
#include <unordered_set>

namespace atm {

#define CUDA_CHECK(x)                                                                                   \
    do {                                                                                                \
        cudaError_t err__ = (x);                                                                        \
        if (err__ != cudaSuccess)                                                                       \
            throw Error(4, std::string("CUDA error: ") + cudaGetErrorString(err__) + " at " #x);        \
    } while (0)
#define CUFFT_CHECK(x)                                                                                  \
    do {                                                                                                \
        cufftResult r__ = (x);                                                                          \
        if (r__ != CUFFT_SUCCESS) throw Error(4, std::string("cuFFT error ") + std::to_string((int)r__)); \
    } while (0)

static const double kOne4PiEps0 = 138.935456;  // kJ mol^-1 nm e^-2 (OpenMM 7.x)
static const double kPi = 3.14159265358979323846;

ReplicaSpec spec_from_system(const System& sys) {
    if (!sys.nonbonded) throw Error(5, "The system has no NonbondedForce");
    if (!sys.atm) throw Error(5, "The system has no ATMMetaForce");
    const NonbondedForce& nb = *sys.nonbonded;
    const ATMMetaForce& f = *sys.atm;
    int n = (int)sys.masses.size();
    if ((int)nb.charge.size() != n) throw Error(1, "NonbondedForce particle count differs from the System's");
    if (f.getNumParticles() != n)
        throw Error(9, "ATMMetaForce must hold every System particle (ATMMetaForce.h:94-104)");
    // ATMMetaForceImpl.cpp:75-81
    for (int g : f.groups) {
        if (g == f.forceGroup) throw Error(8, "The ATM Meta Force group cannot be one of the variable force groups.");
        if (g < 0 || g > 31) throw Error(1, "Variable force groups must be between 0 and 31");
    }
    ReplicaSpec s;
    s.n = n;
    s.q = nb.charge;
    s.sig = nb.sigma;
    s.eps = nb.epsilon;
    s.exc = nb.exceptions;
    s.displ.resize(3 * (size_t)n);
    // displacement indexed by the force's particle index (ReferenceATMMetaForceKernels.cpp:121-123)
    for (int i = 0; i < n; i++) {
        s.displ[3 * i] = f.particles[i].dx;
        s.displ[3 * i + 1] = f.particles[i].dy;
        s.displ[3 * i + 2] = f.particles[i].dz;
    }
    s.method = nb.method;
    s.cutoff = nb.cutoff;
    s.epsRF = nb.epsRF;
    s.dispersion = nb.dispersionCorrection;
    for (int a = 0; a < 3; a++) {
        s.box[a] = sys.box[a];
        s.tilt[a] = sys.tilt[a];
    }
    if (nb.method == NonbondedForce::PME) {
        if (nb.alpha > 0 && nb.grid[0] > 0 && nb.grid[1] > 0 && nb.grid[2] > 0) {
            s.alpha = nb.alpha;
            for (int a = 0; a < 3; a++) s.grid[a] = nb.grid[a];
        } else {
            pme_parameters(nb.cutoff, nb.ewaldTol, sys.box, s.alpha, s.grid);
            if (nb.alpha > 0) s.alpha = nb.alpha;
        }
    }
    for (int k = 0; k < NUM_GLOBALS; k++) s.params[k] = f.defaults[k];
    s.var_nb = false;
    for (int g : f.groups)
        if (g == nb.forceGroup) s.var_nb = true;
    return s;
}

// ---------------------------------------------------------------------------
// 3D Hilbert index (J. Skilling, "Programming the Hilbert curve", AIP Conf.
// Proc. 707, 381 (2004): axes -> transposed index, then bit interleave)
// ---------------------------------------------------------------------------
static uint64_t hilbert3(uint32_t x, uint32_t y, uint32_t z, int bits) {
    uint32_t X[3] = {x, y, z};
    uint32_t M = 1u << (bits - 1);
    for (uint32_t Q = M; Q > 1; Q >>= 1) {
        uint32_t P = Q - 1;
        for (int i = 0; i < 3; i++) {
            if (X[i] & Q) {
                X[0] ^= P;
            } else {
                uint32_t t = (X[0] ^ X[i]) & P;
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    for (int i = 1; i < 3; i++) X[i] ^= X[i - 1];
    uint32_t t = 0;
    for (uint32_t Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    for (int i = 0; i < 3; i++) X[i] ^= t;
    uint64_t h = 0;
    for (int b = bits - 1; b >= 0; b--)
        for (int i = 0; i < 3; i++) h = (h << 1) | ((X[i] >> b) & 1u);
    return h;
}

// |sum_{k=0}^{3} M5(k+1) e^{2 pi i m k / K}|^2 with the mean-of-neighbours repair
static void bspline_moduli(int K, std::vector<double>& mod) {
    const double c[4] = {1.0 / 24.0, 11.0 / 24.0, 11.0 / 24.0, 1.0 / 24.0};  // M5(1..4)
    mod.assign(K, 0.0);
    for (int m = 0; m < K; m++) {
        double sc = 0, ss = 0;
        for (int k = 0; k < 4; k++) {
            double arg = 2.0 * kPi * m * k / K;
            sc += c[k] * std::cos(arg);
            ss += c[k] * std::sin(arg);
        }
        mod[m] = sc * sc + ss * ss;
    }
    std::vector<double> fixed = mod;
    for (int m = 0; m < K; m++)
        if (mod[m] < 1e-7) fixed[m] = 0.5 * (mod[(m - 1 + K) % K] + mod[(m + 1) % K]);
    mod = fixed;
}

static double dispersion_coefficient(const ReplicaSpec& s) {
    // 8 pi N^2 (<eps sig^12>/(9 rc^9) - <eps sig^6>/(3 rc^3)), averages over all
    // particle pairs (self pairs included) grouped by (sigma, epsilon) class
    std::map<std::pair<double, double>, double> cls;
    for (int i = 0; i < s.n; i++) cls[{s.sig[i], s.eps[i]}] += 1.0;
    std::vector<std::pair<std::pair<double, double>, double>> v(cls.begin(), cls.end());
    double sum1 = 0, sum2 = 0;
    for (size_t a = 0; a < v.size(); a++)
        for (size_t b = a; b < v.size(); b++) {
            double sig = 0.5 * (v[a].first.first + v[b].first.first);
            double eps = std::sqrt(v[a].first.second * v[b].first.second);
            double cnt = (a == b) ? v[a].second * (v[a].second + 1) / 2 : v[a].second * v[b].second;
            double s6 = std::pow(sig, 6.0);
            sum1 += cnt * eps * s6 * s6;
            sum2 += cnt * eps * s6;
        }
    double N = s.n;
    double np = N * (N + 1) / 2;
    sum1 /= np;
    sum2 /= np;
    return 8.0 * kPi * N * N * (sum1 / (9.0 * std::pow(s.cutoff, 9)) - sum2 / (3.0 * std::pow(s.cutoff, 3)));
}

Engine::Engine(std::vector<ReplicaSpec> reps, int device, bool full_mode, bool adjoint)
    : R_((int)reps.size()), dev_(device), full_(full_mode), adjoint_(adjoint), specs_(std::move(reps)) {
    if (R_ <= 0) throw Error(1, "At least one replica is required");
    if (adjoint_ && full_) throw Error(5, "The adjoint requires the difference path (DifferencePath=1)");
    const ReplicaSpec& s0 = specs_[0];
    method_ = s0.method;
    cutoff_ = s0.cutoff;
    if (method_ < NonbondedForce::NoCutoff || method_ > NonbondedForce::PME)
        throw Error(5, "Unknown nonbonded method");
    if (method_ == 3) throw Error(5, "Plain Ewald summation is not implemented on the GPU path; use PME");
    periodic_ = method_ == NonbondedForce::CutoffPeriodic || method_ == NonbondedForce::PME;
    in_off_.resize(R_);
    for (int r = 0; r < R_; r++) {
        const ReplicaSpec& s = specs_[r];
        if (s.n <= 0) throw Error(1, "Empty replica");
        if (s.method != method_ || s.cutoff != cutoff_ || s.epsRF != s0.epsRF || s.alpha != s0.alpha)
            throw Error(5, "All replicas of a batch must share the nonbonded method, cutoff and Ewald parameters");
        if (periodic_)
            for (int a = 0; a < 3; a++)
                if (!(s.box[a] >= 2.0 * s.cutoff))
                    throw Error(1, "The periodic box must be at least twice the cutoff in every dimension");
        if (s.method == NonbondedForce::PME)
            for (int a = 0; a < 3; a++)
                if (s.grid[a] < 6 || s.grid[a] > 1023)
                    // (the spreading kernels pack a stencil's grid indices in 10 bits each)
                    throw Error(1, "PME grid dimensions must be between 6 and 1023");
        for (const Exception& e : s.exc)
            if (e.i < 0 || e.j < 0 || e.i >= s.n || e.j >= s.n || e.i == e.j)
                throw Error(2, "Exception particle index out of range");
        in_off_[r] = n_in_;
        n_in_ += s.n;
    }
    alpha_ = s0.alpha;
    double er = s0.epsRF;
    if (method_ == NonbondedForce::NoCutoff) {
        krf_ = crf_ = 0.0;  // plain Coulomb, every pair
    } else {
        krf_ = (er - 1.0) / ((2.0 * er + 1.0) * cutoff_ * cutoff_ * cutoff_);
        crf_ = 3.0 * er / ((2.0 * er + 1.0) * cutoff_);
    }

    CUDA_CHECK(cudaSetDevice(dev_));
    CUDA_CHECK(cudaStreamCreateWithFlags(&s_main_, cudaStreamNonBlocking));
    CUDA_CHECK(cudaStreamCreateWithFlags(&s_pme_, cudaStreamNonBlocking));
    CUDA_CHECK(cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming));
    CUDA_CHECK(cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming));
    CUDA_CHECK(cudaEventCreateWithFlags(&ev_fork2_, cudaEventDisableTiming));
    CUDA_CHECK(cudaEventCreateWithFlags(&ev_join2_, cudaEventDisableTiming));
    CUDA_CHECK(cudaMallocHost(&h_pos_, sizeof(double) * 3 * (size_t)n_in_));
    CUDA_CHECK(cudaMallocHost(&h_forces_, sizeof(double) * 3 * (size_t)n_in_));
    CUDA_CHECK(cudaMallocHost(&h_fnb_, sizeof(double) * 3 * (size_t)n_in_));
    CUDA_CHECK(cudaMallocHost(&h_results_, sizeof(double) * NUM_RES * (size_t)R_));
    CUDA_CHECK(cudaMallocHost(&h_matrix_, sizeof(double) * (size_t)R_ * R_));
    // parameter block: ctl (2 ints) at 0, io (3 pointers) at 8, beta at 32, the
    // replica table at kParamReps
    param_bytes_ = kParamReps + sizeof(RepDev) * (size_t)R_;
    CUDA_CHECK(cudaMallocHost(&h_params_, param_bytes_));
    std::memset(h_params_, 0, param_bytes_);
    h_ctl_ = reinterpret_cast<int*>(h_params_);
    h_io_ = reinterpret_cast<double**>(h_params_ + 8);
    h_beta_ = reinterpret_cast<double*>(h_params_ + 32);
    h_reps_ = reinterpret_cast<RepDev*>(h_params_ + kParamReps);
    h_io_[0] = h_io_[1] = h_io_[2] = nullptr;
    CUDA_CHECK(cudaMalloc(&d_counts_, 2 * sizeof(long long)));
    CUDA_CHECK(cudaMemset(d_counts_, 0, 2 * sizeof(long long)));
    h_ctl_[0] = 1;
    h_ctl_[1] = 0;
    CUDA_CHECK(cudaMallocHost(&h_status_, sizeof(Status)));
    std::memset(h_pos_, 0, sizeof(double) * 3 * (size_t)n_in_);
    int per = 0;
    CUDA_CHECK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, dev_));
    per = tiles_kernel_blocks_per_sm();
    if (per < 1) per = 1;
    max_tile_per_sm_ = per;
    tile_grid_ = sms_ * per;
}

Engine::~Engine() {
    cudaSetDevice(dev_);
    if (s_main_) cudaStreamSynchronize(s_main_);
    destroy_graphs();
    free_device();
    for (auto& g : groups_) {
        if (g.fwd) cufftDestroy(g.fwd);
        if (g.inv) cufftDestroy(g.inv);
    }
    cudaFreeHost(h_pos_);
    cudaFreeHost(h_forces_);
    cudaFreeHost(h_fnb_);
    cudaFreeHost(h_results_);
    cudaFreeHost(h_matrix_);
    cudaFreeHost(h_params_);
    if (d_counts_) cudaFree(d_counts_);
    cudaFreeHost(h_status_);
    if (ev_fork_) cudaEventDestroy(ev_fork_);
    if (ev_join_) cudaEventDestroy(ev_join_);
    if (ev_fork2_) cudaEventDestroy(ev_fork2_);
    if (ev_join2_) cudaEventDestroy(ev_join2_);
    if (s_main_) cudaStreamDestroy(s_main_);
    if (s_pme_) cudaStreamDestroy(s_pme_);
}

void Engine::destroy_graphs() {
    if (graph_host_) cudaGraphExecDestroy(graph_host_);
    if (graph_dev_) cudaGraphExecDestroy(graph_dev_);
    if (graph_res_) cudaGraphExecDestroy(graph_res_);
    graph_host_ = graph_dev_ = graph_res_ = nullptr;
}

void Engine::set_positions(int r, const double* pos) {
    if (r < 0 || r >= R_) throw Error(2, "Replica index out of range");
    std::memcpy(h_pos_ + 3 * (size_t)in_off_[r], pos, sizeof(double) * 3 * (size_t)specs_[r].n);
}

void Engine::set_all_positions(const double* pos) {
    std::memcpy(h_pos_, pos, sizeof(double) * 3 * (size_t)n_in_);
}

void Engine::set_box(int r, const double* box, const double* tilt) {
    if (r < 0 || r >= R_) throw Error(2, "Replica index out of range");
    if (periodic_)
        for (int a = 0; a < 3; a++)
            if (!(box[a] >= 2.0 * (cutoff_ + skin_)))
                throw Error(1,
                            "The periodic box must be at least twice the cutoff (plus the list skin) in every dimension");
    for (int a = 0; a < 3; a++) {
        specs_[r].box[a] = box[a];
        specs_[r].tilt[a] = tilt ? tilt[a] : 0.0;
    }
    force_build_ = true;  // periodic images move with the box
    infl_dirty_ = true;
}

void Engine::update_influence(cudaStream_t st) {
    if (!infl_dirty_) return;
    infl_dirty_ = false;
    if (!use_fft_ || method_ != NonbondedForce::PME) return;
    for (int r = 0; r < R_; r++) {
        const RepDev& rd = rep_host_[r];
        const ReplicaSpec& s = specs_[r];
        double rb[6];
        recip_box(s, rb);
        launch_influence(A_.influence + rd.cplx_off / 2, A_.moduli, rd.mod_off, rd.K, rb,
                         s.box[0] * s.box[1] * s.box[2], alpha_, st);
    }
    CUDA_CHECK(cudaGetLastError());
}

void Engine::set_list_skin(double skin) {
    if (!(skin >= 0.0) || skin > 0.5) throw Error(1, "The list skin must lie in [0, 0.5] nm");
    if (periodic_)
        for (int r = 0; r < R_; r++)
            for (int a = 0; a < 3; a++)
                if (!(specs_[r].box[a] >= 2.0 * (cutoff_ + skin)))
                    throw Error(1, "The periodic box must be at least twice the cutoff plus the list skin");
    if (skin == skin_) return;
    skin_ = skin;
    A_.rcl2 = list_cutoff2();
    A_.skin_half2 = (float)(0.25 * skin_ * skin_);
    force_build_ = true;
    destroy_graphs();  // the kernels' arguments are part of the graphs
}

void Engine::set_param(int r, int which, double v) {
    if (r < 0 || r >= R_) throw Error(2, "Replica index out of range");
    if (which < 0 || which >= NUM_GLOBALS) throw Error(2, "Unknown global parameter");
    specs_[r].params[which] = v;
}

void Engine::set_displacements(int r, const double* displ) {
    if (r < 0 || r >= R_) throw Error(2, "Replica index out of range");
    ReplicaSpec& s = specs_[r];
    bool same_classes = true;
    for (int i = 0; i < s.n && same_classes; i++) {
        for (int a = 0; a < 3; a++)
            if (displ[3 * i + a] != s.displ[3 * i + a]) same_classes = false;
    }
    if (same_classes) return;
    std::memcpy(s.displ.data(), displ, sizeof(double) * 3 * (size_t)s.n);
    // the moving set or its displacement changed: rebuild the layout lazily
    layout_ready_ = false;
}

// Box constants of a replica.  Without periodic boundaries the inverse box is 0,
// which makes every minimum image and every wrap the identity (d - L rint(0) = d),
// and the box 1e30 nm, so that no pair is ever taken to need its own image.
void Engine::set_box_constants(RepDev& rd, const ReplicaSpec& s) const {
    for (int a = 0; a < 3; a++) {
        const double L = periodic_ ? s.box[a] : 1.0e30;
        rd.box[a] = (float)L;
        rd.ibox[a] = periodic_ ? (float)(1.0 / L) : 0.0f;
        rd.boxd[a] = L;
        rd.iboxd[a] = periodic_ ? 1.0 / L : 0.0;
        const double t = periodic_ ? s.tilt[a] : 0.0;
        rd.tiltd[a] = t;
        rd.tilt[a] = (float)t;
    }
    rd.tiltd[3] = 0.0;
    rd.tilt[3] = 0.0f;
    rd.tric = (rd.tiltd[0] != 0.0 || rd.tiltd[1] != 0.0 || rd.tiltd[2] != 0.0) ? 1 : 0;
    double r[6];
    recip_box(s, r);
    for (int k = 0; k < 6; k++) rd.recip[k] = periodic_ ? (float)r[k] : 0.0f;
    rd.recip[6] = rd.recip[7] = 0.0f;
    rd.wmin = periodic_ ? (float)min_face_distance(s) : 1.0e30f;
}

// Reciprocal box of a replica (rows, lower triangular): r00, r10, r11, r20, r21,
// r22; the fractional coordinate along box vector d of p is sum_i p_i r[i][d].
void Engine::recip_box(const ReplicaSpec& s, double* r) {
    const double ax = s.box[0], by = s.box[1], cz = s.box[2];
    const double bx = s.tilt[0], cx = s.tilt[1], cy = s.tilt[2];
    r[0] = 1.0 / ax;
    r[1] = -bx / (ax * by);
    r[2] = 1.0 / by;
    r[3] = (bx * cy - by * cx) / (ax * by * cz);
    r[4] = -cy / (by * cz);
    r[5] = 1.0 / cz;
}

// Smallest distance between opposite faces: V / |b x c|, V / |a x c|, V / |a x b|.
double Engine::min_face_distance(const ReplicaSpec& s) {
    const double ax = s.box[0], by = s.box[1], cz = s.box[2];
    const double bx = s.tilt[0], cx = s.tilt[1], cy = s.tilt[2];
    const double V = ax * by * cz;
    const double bc = std::sqrt(by * cz * by * cz + bx * cz * bx * cz + (bx * cy - by * cx) * (bx * cy - by * cx));
    const double ac = ax * std::sqrt(cy * cy + cz * cz);
    const double ab = ax * by;
    return std::min(V / bc, std::min(V / ac, V / ab));
}

// Squared cutoffs of the pair kernel and of the list builds (NoCutoff: every pair;
// 1e29 nm^2 stays below the 3e30 nm^2 at which padding slots are parked).
float Engine::cutoff2() const {
    return method_ == NonbondedForce::NoCutoff ? 1.0e29f : (float)(cutoff_ * cutoff_);
}
float Engine::list_cutoff2() const {
    return method_ == NonbondedForce::NoCutoff ? 1.0e29f : (float)((cutoff_ + skin_) * (cutoff_ + skin_));
}

// ---------------------------------------------------------------------------
// Layout
// ---------------------------------------------------------------------------

void Engine::build_layout() {
    orig_.clear();
    slot_of_.assign(n_in_, -1);
    block_rep_.clear();
    block_cls_.clear();
    qs_.clear();
    lj_.clear();
    displ_sorted_.clear();
    block_d_.clear();
    masks_.clear();
    exc_ij_.clear();
    exc_p_.clear();
    exc_cta_first_.clear();
    rep_host_.assign(R_, RepDev{});
    const double sqk = std::sqrt(kOne4PiEps0);

    std::vector<std::vector<std::pair<int, int>>> blk_ex;  // per block: (J, mask id) J >= I
    std::vector<std::vector<std::pair<int, int>>> blk_dx;  // per block: cross-class entries
    int slot = 0;
    for (int r = 0; r < R_; r++) {
        const ReplicaSpec& s = specs_[r];
        RepDev& rd = rep_host_[r];
        const double* pos = h_pos_ + 3 * (size_t)in_off_[r];
        // displacement classes, in order of first appearance
        std::vector<int> cls(s.n, 0);
        std::vector<std::array<double, 3>> cls_d(1, {0, 0, 0});
        for (int i = 0; i < s.n; i++) {
            double dx = s.displ[3 * i], dy = s.displ[3 * i + 1], dz = s.displ[3 * i + 2];
            if (dx == 0 && dy == 0 && dz == 0) continue;
            int c = -1;
            for (size_t k = 1; k < cls_d.size(); k++)
                if (cls_d[k][0] == dx && cls_d[k][1] == dy && cls_d[k][2] == dz) c = (int)k;
            if (c < 0) {
                cls_d.push_back({dx, dy, dz});
                c = (int)cls_d.size() - 1;
            }
            cls[i] = c;
        }
        // molecules from the exception graph
        std::vector<int> parent(s.n);
        std::iota(parent.begin(), parent.end(), 0);
        auto find = [&](int x) {
            while (parent[x] != x) {
                parent[x] = parent[parent[x]];
                x = parent[x];
            }
            return x;
        };
        for (const Exception& e : s.exc) {
            int a = find(e.i), b = find(e.j);
            if (a != b) parent[std::max(a, b)] = std::min(a, b);
        }
        // non-moving molecules sorted along a Hilbert curve
        std::map<int, std::vector<int>> mol;
        for (int i = 0; i < s.n; i++)
            if (cls[i] == 0) mol[find(i)].push_back(i);
        std::vector<std::pair<uint64_t, int>> keys;
        const int bits = 10;
        // the cube the curve spans: the periodic box, or the positions' bounding box
        double lo[3] = {0, 0, 0}, span[3] = {s.box[0], s.box[1], s.box[2]};
        if (!periodic_) {
            double hi[3];
            for (int a = 0; a < 3; a++) lo[a] = hi[a] = s.n ? pos[a] : 0.0;
            for (int i = 0; i < s.n; i++)
                for (int a = 0; a < 3; a++) {
                    lo[a] = std::min(lo[a], pos[3 * i + a]);
                    hi[a] = std::max(hi[a], pos[3 * i + a]);
                }
            for (int a = 0; a < 3; a++) span[a] = std::max(hi[a] - lo[a], 1e-6) * (1.0 + 1e-9);
        }
        double rb[6];
        recip_box(s, rb);
        for (auto& kv : mol) {
            int i = kv.second[0];
            uint32_t c[3];
            const double* p = pos + 3 * (size_t)i;
            // periodic: fractional coordinates along the box vectors, wrapped
            const double fr[3] = {p[0] * rb[0] + p[1] * rb[1] + p[2] * rb[3], p[1] * rb[2] + p[2] * rb[4],
                                  p[2] * rb[5]};
            for (int a = 0; a < 3; a++) {
                double x;
                if (periodic_) {
                    x = fr[a] - std::floor(fr[a]);
                } else {
                    x = (p[a] - lo[a]) / span[a];
                }
                long v = (long)(x * (1 << bits));
                c[a] = (uint32_t)std::min(std::max(v, 0L), (long)(1 << bits) - 1);
            }
            keys.push_back({hilbert3(c[0], c[1], c[2], bits), kv.first});
        }
        std::sort(keys.begin(), keys.end());
        std::vector<std::vector<int>> segments(cls_d.size());
        for (auto& k : keys)
            for (int i : mol[k.second]) segments[0].push_back(i);
        for (int i = 0; i < s.n; i++)
            if (cls[i] != 0) segments[cls[i]].push_back(i);

        rd.slot_begin = slot;
        rd.block_begin = slot / kTile;
        rd.mov_block_begin = -1;
        rd.in_off = in_off_[r];
        rd.n = s.n;
        std::vector<int> slot_local(s.n, -1);
        for (size_t c = 0; c < segments.size(); c++) {
            if (segments[c].empty()) continue;
            if (c >= 1 && rd.mov_block_begin < 0) rd.mov_block_begin = slot / kTile;
            for (int i : segments[c]) {
                slot_local[i] = slot;
                slot_of_[in_off_[r] + i] = slot;
                orig_.push_back(i);
                qs_.push_back((float)(s.q[i] * sqk));
                lj_.push_back(make_float2((float)(0.5 * s.sig[i]), (float)(2.0 * std::sqrt(s.eps[i]))));
                displ_sorted_.push_back(make_float4((float)s.displ[3 * i], (float)s.displ[3 * i + 1],
                                                    (float)s.displ[3 * i + 2], 0.f));
                slot++;
            }
            while (slot % kTile) {
                orig_.push_back(-1);
                qs_.push_back(0.f);
                lj_.push_back(make_float2(0.f, 0.f));
                displ_sorted_.push_back(displ_sorted_.back());
                slot++;
            }
        }
        rd.slot_end = slot;
        rd.block_end = slot / kTile;
        if (rd.mov_block_begin < 0) rd.mov_block_begin = rd.block_end;
        for (int b = rd.block_begin; b < rd.block_end; b++) {
            block_rep_.push_back(r);
            int o = orig_[b * kTile];
            int c = cls[o];
            block_cls_.push_back(c);
            block_d_.push_back(make_float4((float)cls_d[c][0], (float)cls_d[c][1], (float)cls_d[c][2], 0.f));
        }
        blk_ex.resize(rd.block_end);
        blk_dx.resize(rd.block_end);

        // exclusion tiles: masks (bit k of word l: pair (l, (l+k)&31) is computed)
        std::map<std::pair<int, int>, int> tile_mask;
        auto get_mask = [&](int bi, int bj) {
            auto it = tile_mask.find({bi, bj});
            if (it != tile_mask.end()) return it->second;
            int id = (int)(masks_.size() / 32);
            masks_.resize(masks_.size() + 32, 0xffffffffu);
            tile_mask[{bi, bj}] = id;
            return id;
        };
        for (int b = rd.block_begin; b < rd.block_end; b++) {
            int id = get_mask(b, b);
            for (int l = 0; l < 32; l++) {
                uint32_t& w = masks_[(size_t)id * 32 + l];
                w &= ~1u;  // self
                bool pl = orig_[b * kTile + l] < 0;
                for (int k = 0; k < 32; k++) {
                    int lj2 = (l + k) & 31;
                    if (pl || orig_[b * kTile + lj2] < 0) w &= ~(1u << k);
                }
            }
        }
        std::map<std::pair<int, int>, int> cross_mask;
        std::unordered_set<uint64_t> seen;
        for (const Exception& e : s.exc) {
            int a = std::min(e.i, e.j), b2 = std::max(e.i, e.j);
            uint64_t key = ((uint64_t)a << 32) | (uint64_t)b2;
            if (!seen.insert(key).second) throw Error(1, "Multiple exceptions are specified for one particle pair");
            int si = slot_local[e.i], sj = slot_local[e.j];
            int bi = si / kTile, bj = sj / kTile, li = si % kTile, lj = sj % kTile;
            if (bi > bj || (bi == bj && li > lj)) {
                std::swap(bi, bj);
                std::swap(li, lj);
            }
            int id = get_mask(bi, bj);
            masks_[(size_t)id * 32 + li] &= ~(1u << ((lj - li) & 31));
            if (bi == bj) masks_[(size_t)id * 32 + lj] &= ~(1u << ((li - lj) & 31));
            // a pair whose atoms move differently is also masked in the difference tiles
            int ci = cls[e.i], cj = cls[e.j];
            if (ci != cj && !full_) {
                int si2 = slot_local[e.i], sj2 = slot_local[e.j];
                // the row belongs to the moving atom with the smaller class (non-moving = 0 never owns a row)
                if (ci == 0 || (cj != 0 && cj < ci)) {
                    std::swap(si2, sj2);
                    std::swap(ci, cj);
                }
                int rbi = si2 / kTile, rbj = sj2 / kTile, rli = si2 % kTile, rlj = sj2 % kTile;
                auto it = cross_mask.find({rbi, rbj});
                int cid;
                if (it == cross_mask.end()) {
                    cid = (int)(masks_.size() / 32);
                    masks_.resize(masks_.size() + 32, 0xffffffffu);
                    cross_mask[{rbi, rbj}] = cid;
                } else {
                    cid = it->second;
                }
                masks_[(size_t)cid * 32 + rli] &= ~(1u << ((rlj - rli) & 31));
            }
        }
        for (auto& kv : tile_mask) blk_ex[kv.first.first].push_back({kv.first.second, kv.second});
        for (auto& kv : cross_mask) blk_dx[kv.first.first].push_back({kv.first.second, kv.second});

        // exceptions, user-order indices
        rd.exc_cta_b = (int)exc_cta_first_.size();
        int first_exc = (int)exc_ij_.size();
        for (const Exception& e : s.exc) {
            bool cross = cls[e.i] != cls[e.j];
            exc_ij_.push_back(make_int4(in_off_[r] + e.i, in_off_[r] + e.j, r, cross ? 1 : 0));
            exc_p_.push_back(ExcParam{e.qq * kOne4PiEps0, e.sig, e.eps, kOne4PiEps0 * s.q[e.i] * s.q[e.j]});
        }
        for (int k = first_exc; k < (int)exc_ij_.size(); k += 256) exc_cta_first_.push_back(k);
        rd.exc_cta_e = (int)exc_cta_first_.size();

        // box and constants
        set_box_constants(rd, s);
        for (int a = 0; a < 3; a++) rd.K[a] = s.grid[a];
        double q2 = 0;
        for (int i = 0; i < s.n; i++) q2 += s.q[i] * s.q[i];
        rd.e_self = (method_ == NonbondedForce::PME) ? -kOne4PiEps0 * alpha_ / std::sqrt(kPi) * q2 : 0.0;
        rd.var_nb = s.var_nb ? 1 : 0;
    }
    exc_cta_first_.push_back((int)exc_ij_.size());
    NA_ = slot;
    NB_ = slot / kTile;

    // exclusion CSR
    ex_start_.assign(NB_ + 1, 0);
    dx_start_.assign(NB_ + 1, 0);
    ex_ent_.clear();
    dx_ent_.clear();
    for (int b = 0; b < NB_; b++) {
        std::sort(blk_ex[b].begin(), blk_ex[b].end());
        std::sort(blk_dx[b].begin(), blk_dx[b].end());
        ex_start_[b] = (int)ex_ent_.size();
        for (auto& e : blk_ex[b]) ex_ent_.push_back(make_int2(e.first, e.second));
        dx_start_[b] = (int)dx_ent_.size();
        for (auto& e : blk_dx[b]) dx_ent_.push_back(make_int2(e.first, e.second));
    }
    ex_start_[NB_] = (int)ex_ent_.size();
    dx_start_[NB_] = (int)dx_ent_.size();
    if (masks_.empty()) masks_.resize(32, 0xffffffffu);

    // The pair-tile kernel works on half blocks (16 x 16 tiles).  Sub-tile (a, b)
    // of exclusion tile (I, J) pairs atoms 16a .. 16a+15 of I with 16b .. 16b+15
    // of J; its mask word l, bit k: pair (l, (l + k) & 15) is computed.  Of a
    // diagonal tile: (0,0) and (1,1) (both orders, as the full tile) and (0,1);
    // sub-tiles without a computed pair are dropped.
    masks16_.clear();
    exs_start_.assign(NB_ + 1, 0);
    dxs_start_.assign(NB_ + 1, 0);
    exs_ent_.clear();
    dxs_ent_.clear();
    auto add_subtiles = [&](int I, int J, int id, std::vector<int4>& out) {
        for (int sa = 0; sa < 2; sa++)
            for (int sb = 0; sb < 2; sb++) {
                if (I == J && sa > sb) continue;
                uint32_t m[kHalf];
                bool any = false;
                for (int l = 0; l < kHalf; l++) {
                    const int ii = kHalf * sa + l;
                    const uint32_t w = masks_[(size_t)id * 32 + ii];
                    uint32_t v = 0;
                    for (int k = 0; k < kHalf; k++) {
                        const int jj = kHalf * sb + ((l + k) & (kHalf - 1));
                        if ((w >> ((jj - ii) & 31)) & 1u) v |= 1u << k;
                    }
                    m[l] = v;
                    any = any || v != 0;
                }
                if (!any) continue;
                const int id16 = (int)(masks16_.size() / kHalf);
                masks16_.insert(masks16_.end(), m, m + kHalf);
                out.push_back(make_int4(2 * I + sa, 2 * J + sb, id16, 0));
            }
    };
    for (int b = 0; b < NB_; b++) {
        exs_start_[b] = (int)exs_ent_.size();
        for (auto& e : blk_ex[b]) add_subtiles(b, e.first, e.second, exs_ent_);
        dxs_start_[b] = (int)dxs_ent_.size();
        for (auto& e : blk_dx[b]) add_subtiles(b, e.first, e.second, dxs_ent_);
    }
    exs_start_[NB_] = (int)exs_ent_.size();
    dxs_start_[NB_] = (int)dxs_ent_.size();
    if (masks16_.empty()) masks16_.resize(kHalf, 0xffffu);

    // rows: all state-1 rows, then state-2 rows (full) or the difference rows
    row_desc_.clear();
    for (int b = 0; b < NB_; b++) row_desc_.push_back(make_int4(b, ROW_STATE1, block_rep_[b], 0));
    for (int r = 0; r < R_; r++) {
        rep_host_[r].row1_b = rep_host_[r].block_begin;
        rep_host_[r].row1_e = rep_host_[r].block_end;
    }
    for (int r = 0; r < R_; r++) {
        RepDev& rd = rep_host_[r];
        rd.row2_b = (int)row_desc_.size();
        if (full_) {
            for (int b = rd.block_begin; b < rd.block_end; b++) row_desc_.push_back(make_int4(b, ROW_STATE2, r, 0));
        } else {
            for (int b = rd.mov_block_begin; b < rd.block_end; b++) {
                row_desc_.push_back(make_int4(b, ROW_DIFF1, r, 0));
                row_desc_.push_back(make_int4(b, ROW_DIFF2, r, 0));
            }
        }
        rd.row2_e = (int)row_desc_.size();
    }
    // Few rows for the finder's resident warps: each row's candidate blocks are
    // split over up to 4 warps (parts: the warps per row, and 2 while the rows are
    // fewer than twice the warps), so that the list building is not the latency of
    // a few long rows (the difference rows scan every block of their replica).
    // Measured on subsets of the 22 x 23,558-atom batch: 4 replicas 11,800 -> 14,300
    // evaluations/s (2 parts instead of 1), 5 replicas 12,400 -> 14,900, 8 replicas
    // 16,400 -> 17,600; two parts at 11 and 22 replicas lost 3-4 %, and 3 parts
    // in place of 2 at 2 replicas lost 4 %.
    {
        const int base_rows = (int)row_desc_.size();
        const int warps = sms_ * find_warps_per_sm();
        int parts = base_rows > 0 ? warps / base_rows : 1;
        if (parts <= 1 && 2 * warps > base_rows) parts = 2;
        parts = std::max(1, std::min(4, parts));
        if (parts > 1) {
            std::vector<int4> split;
            split.reserve((size_t)base_rows * parts);
            for (const int4& d : row_desc_)
                for (int p = 0; p < parts; p++) split.push_back(make_int4(d.x, d.y, d.z, p | (parts << 8)));
            row_desc_.swap(split);
            for (int r = 0; r < R_; r++) {
                RepDev& rd = rep_host_[r];
                rd.row1_b *= parts;
                rd.row1_e *= parts;
                rd.row2_b *= parts;
                rd.row2_e *= parts;
            }
        }
        row_parts_ = parts;
    }
    nrows_ = (int)row_desc_.size();

    // PME grids grouped by dimensions (one batched cuFFT plan per group)
    n_real_ = n_cplx_ = 0;
    moduli_.clear();
    conv_cta_rep_.clear();
    conv_cta_first_.clear();
    for (auto& g : groups_) {
        if (g.fwd) cufftDestroy(g.fwd);
        if (g.inv) cufftDestroy(g.inv);
    }
    groups_.clear();
    fft_tw_.clear();
    fft_stages_.clear();
    fft_plane_.clear();
    fft_conv_.clear();
    use_fft_ = false;
    if (method_ == NonbondedForce::PME) {
        std::vector<int> order(R_);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            const int* a = specs_[x].grid;
            const int* b = specs_[y].grid;
            return std::lexicographical_compare(a, a + 3, b, b + 3);
        });
        for (int r : order) {
            RepDev& rd = rep_host_[r];
            if (groups_.empty() || std::memcmp(groups_.back().K, rd.K, sizeof(rd.K)) != 0) {
                FftGroup g;
                std::memcpy(g.K, rd.K, sizeof(g.K));
                g.first_rep = r;
                g.count = 0;
                g.real_off = n_real_;
                g.cplx_off = n_cplx_;
                groups_.push_back(g);
            }
            groups_.back().count++;
            long long G3 = (long long)rd.K[0] * rd.K[1] * rd.K[2];
            long long C3 = (long long)rd.K[0] * rd.K[1] * (rd.K[2] / 2 + 1);
            rd.real_off = n_real_;
            rd.cplx_off = n_cplx_;
            n_real_ += 2 * G3;
            n_cplx_ += 2 * C3;
            for (int a = 0; a < 3; a++) {
                std::vector<double> m;
                bspline_moduli(rd.K[a], m);
                rd.mod_off[a] = (int)moduli_.size();
                for (double v : m) moduli_.push_back((float)v);
                // FFT twiddles w_N^k = exp(-2 pi i k / N), computed in FP64
                rd.tw_off[a] = (int)fft_tw_.size();
                for (int k = 0; k < rd.K[a]; k++) {
                    const double t = -2.0 * kPi * k / rd.K[a];
                    fft_tw_.push_back(make_float2((float)std::cos(t), (float)std::sin(t)));
                }
                rd.fft_plan[a] = fft_plan_stages(rd.K[a], fft_stages_);
            }
        }
        // the hand-written transforms need a grid plane (two buffers) in shared memory
        int smem_max = 0;
        CUDA_CHECK(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_));
        fft_plane_smem_ = fft_conv_smem_ = 0;
        use_fft_ = true;
        for (int r = 0; r < R_; r++) {
            const RepDev& rd = rep_host_[r];
            const int b = fft_plane_smem_bytes(rd.K[1], rd.K[2]);
            fft_plane_smem_ = std::max(fft_plane_smem_, b);
            if (b > smem_max - 1024) use_fft_ = false;
        }
        for (int r = 0; r < R_; r++) {
            RepDev& rd = rep_host_[r];
            long long C3 = (long long)rd.K[0] * rd.K[1] * (rd.K[2] / 2 + 1);
            rd.conv_cta_b = use_fft_ ? (int)fft_conv_.size() : (int)conv_cta_rep_.size();
            if (use_fft_) {
                for (int g = 0; g < 2; g++)
                    for (int x = 0; x < rd.K[0]; x++) fft_plane_.push_back(make_int2(r, g * rd.K[0] + x));
                // kz chunks of the (x, kz) slab of both grids small enough for two CTAs per SM
                const int K2h = rd.K[2] / 2 + 1;
                int nz = K2h;
                while (nz > 1 && fft_conv_smem_bytes(rd.K[0], nz) > 100 * 1024) nz = (nz + 1) / 2;
                for (int ky = 0; ky < rd.K[1]; ky++)
                    for (int z0 = 0; z0 < K2h; z0 += nz) fft_conv_.push_back(make_int4(r, ky, z0, std::min(K2h, z0 + nz)));
                fft_conv_smem_ = std::max(fft_conv_smem_, fft_conv_smem_bytes(rd.K[0], nz));
                rd.conv_cta_e = (int)fft_conv_.size();
            } else {
                const long long per = 4096;
                for (long long k = 0; k < C3; k += per) {
                    conv_cta_rep_.push_back(r);
                    conv_cta_first_.push_back(k);
                }
                rd.conv_cta_e = (int)conv_cta_rep_.size();
            }
        }
        build_bricks();
    } else {
        for (int r = 0; r < R_; r++) {
            rep_host_[r].conv_cta_b = rep_host_[r].conv_cta_e = 0;
        }
    }
    for (int r = 0; r < R_; r++) {
        const ReplicaSpec& s = specs_[r];
        rep_host_[r].e_disp = 0.0;
        if (s.dispersion && periodic_)
            rep_host_[r].e_disp = dispersion_coefficient(s) / (s.box[0] * s.box[1] * s.box[2]);
    }
    if (tile_cap_ == 0) tile_cap_ = nrows_ * 56 + 8192;
    layout_ready_ = true;
}

// Spreading bricks: at most tune_brick_ grid points per dimension, two grids per
// replica.  Spreading by owner needs the hand-written forward transform (it reads
// the int32 grids) and grids larger than a brick plus the stencil reach (4 points)
// in every dimension of every replica, so that a brick's padded accumulator never
// wraps onto itself.  tune_brick_ 0: spreading per atom (k_spread_atoms, int32
// grids, also with the hand-written transform only; bricks of 16 otherwise).
void Engine::build_bricks() {
    brick_cta_rep_.clear();
    brick_smem_ = 0;
    spread_atoms_ = tune_brick_ == 0 && use_fft_;
    const int edge = tune_brick_ > 0 ? tune_brick_ : 16;
    spread_owner_ = spread_owner_pref_ && use_fft_;
    for (int r = 0; r < R_; r++) {
        RepDev& rd = rep_host_[r];
        for (int d = 0; d < 3; d++) {
            rd.nbrick[d] = (rd.K[d] + edge - 1) / edge;
            rd.bsz[d] = (rd.K[d] + rd.nbrick[d] - 1) / rd.nbrick[d];
            if (rd.K[d] < rd.bsz[d] + kOrder - 1) spread_owner_ = false;
        }
        rd.brick_cta_b = (int)brick_cta_rep_.size();
        int nb = rd.nbrick[0] * rd.nbrick[1] * rd.nbrick[2];
        for (int k = 0; k < 2 * nb; k++) brick_cta_rep_.push_back(r);
    }
    // int32 accumulator of a brick padded by the stencil reach (4 points) below it
    // (by owner) or on each side, z rows at a bank-spreading stride
    const int span = spread_owner_ ? kOrder - 1 : 2 * (kOrder - 1);
    for (int r = 0; r < R_; r++) {
        const RepDev& rd = rep_host_[r];
        brick_smem_ = std::max(brick_smem_, (int)(sizeof(int) * (rd.bsz[0] + span) * (rd.bsz[1] + span) *
                                                  spread_row_stride(rd.bsz[2] + span)));
    }
}

void Engine::set_spread_brick(int brick) {
    if (brick < 0 || (brick > 0 && brick < kOrder)) throw Error(1, "SpreadBrick must be 0 (per atom) or at least 5");
    apply_tuning(tune_tile_per_sm_ > 0 ? tune_tile_per_sm_ : max_tile_per_sm_, brick, tune_pme_stream_, tune_fused_);
}

void Engine::set_spread_owner(bool on) {
    if (on == spread_owner_pref_) return;
    spread_owner_pref_ = on;
    if (layout_ready_ && method_ == NonbondedForce::PME) {
        build_bricks();
        alloc_device();
    }
    destroy_graphs();
}

// ---------------------------------------------------------------------------
// Autotuner: times the evaluation graph over pair-tile residency, spreading
// brick size and PME stream overlap; keeps the fastest (cached per workload).
// ---------------------------------------------------------------------------

std::string Engine::tuning_key() const {
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, dev_);
    std::ostringstream k;
    k << prop.name << "|R" << R_ << "|N" << n_in_ << "|m" << method_ << "|rc" << cutoff_ << "|full" << full_
      << "|adj" << adjoint_;
    if (!rep_host_.empty()) k << "|K" << rep_host_[0].K[0] << "x" << rep_host_[0].K[1] << "x" << rep_host_[0].K[2];
    return k.str();
}

void Engine::apply_tuning(int tile_per_sm, int brick, bool pme_stream, bool fused) {
    bool rebuild = brick != tune_brick_;
    tune_tile_per_sm_ = tile_per_sm;
    tune_brick_ = brick;
    tune_pme_stream_ = pme_stream;
    tune_fused_ = fused;
    A_.fused = fused ? 1 : 0;
    tile_grid_ = sms_ * std::min(std::max(1, tile_per_sm), max_tile_per_sm_);
    A_.tile_dynamic = tile_dynamic();
    A_.tile_wide = tile_grid_ <= 3 * sms_ ? 1 : 0;
    if (rebuild && layout_ready_ && method_ == NonbondedForce::PME) {
        build_bricks();
        alloc_device();
    }
    destroy_graphs();
}

void Engine::set_fused(bool fused) {
    if (fused == tune_fused_) return;
    tune_fused_ = fused;
    A_.fused = fused ? 1 : 0;
    destroy_graphs();
}

static std::string cache_path() {
    const char* p = std::getenv("ATM_AUTOTUNE_CACHE");
    if (p && *p) return p;
    const char* x = std::getenv("XDG_CACHE_HOME");
    const char* h = std::getenv("HOME");
    if (x && *x) return std::string(x) + "/atm_gb300_autotune.txt";
    if (h && *h) return std::string(h) + "/.cache/atm_gb300_autotune.txt";
    return "atm_gb300_autotune.txt";
}

bool Engine::load_tuning() {
    std::ifstream f(cache_path());
    std::string line, key = tuning_key();
    while (std::getline(f, line)) {
        auto tab = line.find('\t');
        if (tab == std::string::npos || line.substr(0, tab) != key) continue;
        std::istringstream v(line.substr(tab + 1));
        int t, b, s, fu = 0;
        if (v >> t >> b >> s) {
            if (!(v >> fu)) fu = 0;
            apply_tuning(t, b, s != 0, fu != 0);
            return true;
        }
    }
    return false;
}

std::string Engine::autotune(int trials, bool use_cache) {
    CUDA_CHECK(cudaSetDevice(dev_));
    if (!layout_ready_) {
        build_layout();
        alloc_device();
    }
    if (use_cache && load_tuning()) return "cached: " + tuning_key();
    std::ostringstream rep;
    double best = 1e30;
    int bt = max_tile_per_sm_, bb = tune_brick_;
    bool bs = tune_pme_stream_, bf = tune_fused_;
    const bool pme = method_ == NonbondedForce::PME;
    // spreading bricks of 20, 19, 16, 12 points, or per atom (0: small systems)
    std::vector<int> bricks = pme ? std::vector<int>{20, 19, 16, 12} : std::vector<int>{tune_brick_};
    if (pme && use_fft_) bricks.push_back(0);
    std::vector<int> pmes = pme ? std::vector<int>{1, 0} : std::vector<int>{1};
    cudaEvent_t e0, e1;
    CUDA_CHECK(cudaEventCreate(&e0));
    CUDA_CHECK(cudaEventCreate(&e1));
    // separate list and pair-tile kernels at 4, 3, 2 pair-tile CTAs per SM, then the
    // fused kernel (its CTAs per SM are fixed)
    std::vector<std::pair<int, bool>> shapes;
    for (int t = max_tile_per_sm_; t >= 2 && t >= max_tile_per_sm_ - 2; t--) shapes.push_back({t, false});
    shapes.push_back({max_tile_per_sm_, true});
    for (const auto& sh : shapes)
        for (int b : bricks)
            for (int s : pmes) {
                const int t = sh.first;
                const bool fu = sh.second;
                apply_tuning(t, b, s != 0, fu);
                run(true, nullptr, nullptr);   // uploads the staged positions (buffers may be new)
                run(false, nullptr, nullptr);  // device graph capture + one warm evaluation
                CUDA_CHECK(cudaEventRecord(e0, s_main_));
                for (int k = 0; k < trials; k++) CUDA_CHECK(cudaGraphLaunch(graph_dev_, s_main_));
                CUDA_CHECK(cudaEventRecord(e1, s_main_));
                CUDA_CHECK(cudaEventSynchronize(e1));
                float ms = 0;
                CUDA_CHECK(cudaEventElapsedTime(&ms, e0, e1));
                ms /= trials;
                if (fu)
                    rep << "fused lists+tiles";
                else
                    rep << "tiles/SM=" << t;
                rep << " brick=" << b << " pme_stream=" << s << " : " << ms << " ms\n";
                if (ms < best) {
                    best = ms;
                    bt = t;
                    bb = b;
                    bs = s != 0;
                    bf = fu;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply_tuning(bt, bb, bs, bf);
    rep << "chosen: " << (bf ? "fused lists+tiles" : "tiles/SM=" + std::to_string(bt)) << " brick=" << bb
        << " pme_stream=" << bs << " (" << best << " ms)\n";
    std::ofstream f(cache_path(), std::ios::app);
    if (f) f << tuning_key() << "\t" << bt << " " << bb << " " << (bs ? 1 : 0) << " " << (bf ? 1 : 0) << "\n";
    return rep.str();
}

// ---------------------------------------------------------------------------
// Device buffers
// ---------------------------------------------------------------------------

void Engine::free_device() {
    for (void* p : d_allocs_) cudaFree(p);
    d_allocs_.clear();
}

template <typename T>
static T* dalloc(std::vector<void*>& list, size_t n) {
    void* p = nullptr;
    if (n == 0) n = 1;
    CUDA_CHECK(cudaMalloc(&p, n * sizeof(T)));
    list.push_back(p);
    return (T*)p;
}

template <typename T>
static T* dupload(std::vector<void*>& list, const std::vector<T>& v) {
    T* p = dalloc<T>(list, v.size());
    if (!v.empty()) CUDA_CHECK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

void Engine::alloc_device() {
    CUDA_CHECK(cudaSetDevice(dev_));
    destroy_graphs();
    free_device();
    Args& a = A_;
    a = Args{};
    a.R = R_;
    a.NA = NA_;
    a.NB = NB_;
    a.nrows = nrows_;
    a.row_cap = row_cap_;
    a.tile_cap = tile_cap_;
    a.n_in = n_in_;
    a.full = full_ ? 1 : 0;
    a.method = method_;
    a.rc2 = cutoff2();
    a.rcl2 = list_cutoff2();
    a.skin_half2 = (float)(0.25 * skin_ * skin_);
    a.tile_dynamic = tile_dynamic();
    a.tile_wide = tile_grid_ <= 3 * sms_ ? 1 : 0;
    a.fused = tune_fused_ ? 1 : 0;
    a.alpha = (float)alpha_;
    a.krf = (float)krf_;
    a.crf = (float)crf_;
    a.alphad = alpha_;
    a.cutoffd = cutoff_;
    d_params_ = dalloc<char>(d_allocs_, param_bytes_);
    CUDA_CHECK(cudaMemset(d_params_, 0, param_bytes_));
    a.reps = reinterpret_cast<RepDev*>(d_params_ + kParamReps);
    a.pos_in = dalloc<double>(d_allocs_, 3 * (size_t)n_in_);
    {
        std::vector<double> d(3 * (size_t)n_in_);
        for (int r = 0; r < R_; r++)
            std::memcpy(d.data() + 3 * (size_t)in_off_[r], specs_[r].displ.data(), sizeof(double) * 3 * specs_[r].n);
        a.displ_in = dupload(d_allocs_, d);
    }
    a.slot_of = dupload(d_allocs_, slot_of_);
    a.f_out = dalloc<double>(d_allocs_, 3 * (size_t)n_in_);
    a.io = reinterpret_cast<double**>(d_params_ + 8);
    a.f_nb = dalloc<double>(d_allocs_, 3 * (size_t)n_in_);
    a.orig = dupload(d_allocs_, orig_);
    a.qs = dupload(d_allocs_, qs_);
    a.lj = dupload(d_allocs_, lj_);
    a.displ = dupload(d_allocs_, displ_sorted_);
    a.posq = dalloc<float4>(d_allocs_, NA_);
    a.posq2 = full_ ? dalloc<float4>(d_allocs_, NA_) : nullptr;
    a.posq_ref = dalloc<float4>(d_allocs_, NA_);
    a.rep_hmax = dalloc<unsigned>(d_allocs_, R_);
    a.list_counts = d_counts_;
    a.list_ctl = reinterpret_cast<int*>(d_params_);
    force_build_ = true;  // new buffers hold no lists
    a.block_rep = dupload(d_allocs_, block_rep_);
    a.block_cls = dupload(d_allocs_, block_cls_);
    a.block_d = dupload(d_allocs_, block_d_);
    {
        std::vector<int> mov;
        for (int b = 0; b < NB_; b++)
            if (block_cls_[b] != 0) mov.push_back(b);
        a.n_mov_blocks = (int)mov.size();
        a.mov_blocks = dupload(d_allocs_, mov);
    }
    a.bb_c = dalloc<float4>(d_allocs_, NB_);
    a.bb_h = dalloc<float4>(d_allocs_, NB_);
    a.bb_c2 = full_ ? dalloc<float4>(d_allocs_, NB_) : nullptr;
    a.bb_h2 = full_ ? dalloc<float4>(d_allocs_, NB_) : nullptr;
    a.row_desc = dupload(d_allocs_, row_desc_);
    a.row_count = dalloc<int>(d_allocs_, nrows_);
    a.row_tbase = dalloc<int>(d_allocs_, nrows_);
    a.ex_start = dupload(d_allocs_, ex_start_);
    a.ex_ent = dupload(d_allocs_, ex_ent_);
    a.dx_start = dupload(d_allocs_, dx_start_);
    a.dx_ent = dupload(d_allocs_, dx_ent_);
    a.masks = dupload(d_allocs_, masks16_);
    a.exs_start = dupload(d_allocs_, exs_start_);
    a.exs_ent = dupload(d_allocs_, exs_ent_);
    a.dxs_start = dupload(d_allocs_, dxs_start_);
    a.dxs_ent = dupload(d_allocs_, dxs_ent_);
    a.tiles = dalloc<int4>(d_allocs_, tile_cap_);
    a.tile_j = dalloc<int>(d_allocs_, (size_t)kHalf * tile_cap_);
    a.e_tile = dalloc<float2>(d_allocs_, (size_t)nrows_ * row_cap_);
    {
        // finalize: about 32 rows per CTA, at most 64 CTAs per replica
        int rows = 1;
        for (int r = 0; r < R_; r++)
            rows = std::max(rows, (rep_host_[r].row1_e - rep_host_[r].row1_b) + (rep_host_[r].row2_e - rep_host_[r].row2_b));
        a.fin_ctas = std::min(64, std::max(1, (rows + 31) / 32));
        a.fin_part = dalloc<double>(d_allocs_, (size_t)R_ * a.fin_ctas * 2);
        a.fin_count = dalloc<int>(d_allocs_, (size_t)R_);
        CUDA_CHECK(cudaMemset(a.fin_count, 0, sizeof(int) * (size_t)R_));
    }
    a.status = dalloc<Status>(d_allocs_, 1);
    a.F = dalloc<unsigned long long>(d_allocs_, 6 * (size_t)NA_);
    a.adjoint = adjoint_ ? 1 : 0;
    a.D = adjoint_ ? dalloc<unsigned long long>(d_allocs_, 3 * (size_t)NA_) : nullptr;
    a.sqrt_ke = std::sqrt(kOne4PiEps0);
    a.n_exc = (int)exc_ij_.size();
    a.exc_ij = dupload(d_allocs_, exc_ij_);
    a.exc_p = dupload(d_allocs_, exc_p_);
    a.exc_ctas = (int)exc_cta_first_.size() - 1;
    a.exc_cta_first = dupload(d_allocs_, exc_cta_first_);
    a.e_part_exc = dalloc<double>(d_allocs_, 3 * (size_t)std::max(1, a.exc_ctas));
    a.n_real_total = n_real_;
    if (method_ == NonbondedForce::PME) {
        a.brick_ctas = (int)brick_cta_rep_.size();
        a.brick_smem = brick_smem_;
        a.spread_owner = spread_owner_ || spread_atoms_ ? 1 : 0;
        a.spread_atoms = spread_atoms_ ? 1 : 0;
        a.brick_cta_rep = dupload(d_allocs_, brick_cta_rep_);
        a.qreal = dalloc<float>(d_allocs_, n_real_);
        a.qcplx = dalloc<float2>(d_allocs_, n_cplx_);
        a.moduli = dupload(d_allocs_, moduli_);
        a.use_fft = use_fft_ ? 1 : 0;
        a.fft_tw = dupload(d_allocs_, fft_tw_);
        a.fft_stages = dupload(d_allocs_, fft_stages_);
        a.fft_plane_ctas = (int)fft_plane_.size();
        a.fft_plane = dupload(d_allocs_, fft_plane_);
        a.fft_plane_smem = fft_plane_smem_;
        a.fft_conv = dupload(d_allocs_, fft_conv_);
        a.fft_conv_smem = fft_conv_smem_;
        a.influence = use_fft_ ? dalloc<float>(d_allocs_, n_cplx_ / 2) : nullptr;
        infl_dirty_ = true;
        a.conv_ctas = use_fft_ ? (int)fft_conv_.size() : (int)conv_cta_rep_.size();
        a.conv_cta_rep = dupload(d_allocs_, conv_cta_rep_);
        // per-CTA [first, last) element ranges within each replica's spectrum
        std::vector<long long> pairs(2 * conv_cta_rep_.size());
        for (size_t c = 0; c < conv_cta_rep_.size(); c++) {
            int r = conv_cta_rep_[c];
            const RepDev& rd = rep_host_[r];
            long long C3 = (long long)rd.K[0] * rd.K[1] * (rd.K[2] / 2 + 1);
            bool last = (c + 1 == conv_cta_rep_.size()) || conv_cta_rep_[c + 1] != r;
            pairs[2 * c] = conv_cta_first_[c];
            pairs[2 * c + 1] = last ? C3 : conv_cta_first_[c + 1];
        }
        a.conv_cta_first = dupload(d_allocs_, pairs);
        a.e_part_conv = dalloc<double>(d_allocs_, 2 * (size_t)std::max(1, a.conv_ctas));
        for (auto& g : groups_) {
            if (use_fft_) break;  // library plans only for grids beyond the hand-written transforms
            int n[3] = {g.K[0], g.K[1], g.K[2]};
            long long G3 = (long long)n[0] * n[1] * n[2];
            long long C3 = (long long)n[0] * n[1] * (n[2] / 2 + 1);
            CUFFT_CHECK(cufftPlanMany(&g.fwd, 3, n, nullptr, 1, (int)G3, nullptr, 1, (int)C3, CUFFT_R2C, 2 * g.count));
            CUFFT_CHECK(cufftPlanMany(&g.inv, 3, n, nullptr, 1, (int)C3, nullptr, 1, (int)G3, CUFFT_C2R, 2 * g.count));
            CUFFT_CHECK(cufftSetStream(g.fwd, s_pme_));
            CUFFT_CHECK(cufftSetStream(g.inv, s_pme_));
        }
    } else {
        a.conv_ctas = 0;
    }
    a.results = dalloc<double>(d_allocs_, (size_t)R_ * NUM_RES);
    a.matrix = dalloc<double>(d_allocs_, (size_t)R_ * R_);
    a.beta = reinterpret_cast<double*>(d_params_ + 32);
    CUDA_CHECK(cudaMemset(a.status, 0, sizeof(Status)));
}

void Engine::update_rep_table() {
    for (int r = 0; r < R_; r++) {
        RepDev& rd = rep_host_[r];
        const ReplicaSpec& s = specs_[r];
        set_box_constants(rd, s);
        for (int k = 0; k < NUM_GLOBALS; k++) rd.params[k] = s.params[k];
        rd.e_disp = s.dispersion && periodic_ ? dispersion_coefficient(s) / (s.box[0] * s.box[1] * s.box[2]) : 0.0;
    }
    std::memcpy(h_reps_, rep_host_.data(), sizeof(RepDev) * (size_t)R_);
    *h_beta_ = beta_;
    // the finder's variant (orthorhombic or triclinic) is part of the recorded graphs
    int tric = 0;
    for (int r = 0; r < R_; r++) tric |= rep_host_[r].tric;
    if (tric != A_.any_tric) {
        A_.any_tric = tric;
        destroy_graphs();
    }
}

// ---------------------------------------------------------------------------
// One evaluation: the kernel sequence (captured once into a CUDA graph)
// ---------------------------------------------------------------------------

// Hand the pair tiles out from a counter when the warps of the tile kernel get
// many tiles each (about 15 tiles per row); a few per warp go in a fixed stride.
int Engine::tile_dynamic() const {
    const long long warps = (long long)tile_grid_ * (kTileThreads / 32);
    return (long long)nrows_ * 15 >= 16 * warps ? 1 : 0;
}

int Engine::launches_per_eval() const {
    // prepare, decide, find and tiles (or the fused kernel), exceptions, finalize
    // (with the row sums), output, matrix (+ PME kernels)
    int n = tune_fused_ ? 7 : 8;
    // spread, gather (moving atoms included) and the transforms: three of ours
    // (zy, x + convolution, inverse yz), or the convolution between library ones
    if (method_ == NonbondedForce::PME) n += use_fft_ ? 5 : 3;
    return n;
}

void Engine::record(cudaStream_t st, int mode) {
    const Args& a = A_;
    const bool host_io = mode == 1;
    if (host_io) {
        CUDA_CHECK(cudaMemcpyAsync((void*)a.pos_in, h_pos_, sizeof(double) * 3 * (size_t)n_in_,
                                   cudaMemcpyHostToDevice, st));
    }
    CUDA_CHECK(cudaMemcpyAsync(d_params_, h_params_, param_bytes_, cudaMemcpyHostToDevice, st));
    CUDA_CHECK(cudaMemsetAsync(a.rep_hmax, 0, sizeof(unsigned) * (size_t)R_, st));
    launch_prepare(a, st);
    launch_decide(a, st);
    bool pme = method_ == NonbondedForce::PME;
    if (pme) {
        // the PME chain on its own stream (overlapping the pair tiles) or in line,
        // as the autotuner chose
        cudaStream_t ps = tune_pme_stream_ ? s_pme_ : st;
        if (tune_pme_stream_) {
            CUDA_CHECK(cudaEventRecord(ev_fork_, st));
            CUDA_CHECK(cudaStreamWaitEvent(s_pme_, ev_fork_, 0));
        }
        // the exceptions need neither lists nor grids: they go first on this
        // stream, beside the list building
        launch_exceptions(a, ps);
        launch_spread(a, ps);
        pme_transforms(ps);
        launch_gather(a, ps);
        if (tune_pme_stream_) CUDA_CHECK(cudaEventRecord(ev_join_, s_pme_));
    }
    if (a.fused) {
        launch_find_tiles(a, st);
    } else {
        launch_find(a, st);
        launch_tiles(a, tile_grid_, st);
    }
    if (!pme) launch_exceptions(a, st);
    if (pme && tune_pme_stream_) CUDA_CHECK(cudaStreamWaitEvent(st, ev_join_, 0));
    launch_finalize(a, st);
    if (pme && tune_pme_stream_) {
        // the R x R matrix beside the force output
        CUDA_CHECK(cudaEventRecord(ev_fork2_, st));
        CUDA_CHECK(cudaStreamWaitEvent(s_pme_, ev_fork2_, 0));
        launch_matrix(a, s_pme_);
        CUDA_CHECK(cudaEventRecord(ev_join2_, s_pme_));
        launch_output(a, st);
        CUDA_CHECK(cudaStreamWaitEvent(st, ev_join2_, 0));
    } else {
        launch_output(a, st);
        launch_matrix(a, st);
    }
    // host flavours: the result records and the R x R matrix (a few KB) end the
    // evaluation in page-locked host memory, so that a host caller needs no copy after it
    if (mode != 0) {
        CUDA_CHECK(cudaMemcpyAsync(h_results_, a.results, sizeof(double) * NUM_RES * (size_t)R_,
                                   cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaMemcpyAsync(h_matrix_, a.matrix, sizeof(double) * (size_t)R_ * R_, cudaMemcpyDeviceToHost,
                                   st));
    }
    if (host_io) {
        CUDA_CHECK(cudaMemcpyAsync(h_forces_, a.f_out, sizeof(double) * 3 * (size_t)n_in_, cudaMemcpyDeviceToHost,
                                   st));
        CUDA_CHECK(cudaMemcpyAsync(h_fnb_, a.f_nb, sizeof(double) * 3 * (size_t)n_in_, cudaMemcpyDeviceToHost, st));
    }
    CUDA_CHECK(cudaMemcpyAsync(h_status_, a.status, sizeof(Status), cudaMemcpyDeviceToHost, st));
}

// Charge grids -> potential grids: the hand-written transforms with the
// convolution fused in, or (grid planes beyond shared memory) the library's R2C,
// the convolution kernel and the library's C2R.  mark(name), when given, follows
// each step (profiling).
void Engine::pme_transforms(cudaStream_t st, const std::function<void(const char*)>& mark) {
    const Args& a = A_;
    if (use_fft_) {
        launch_fft_forward(a, st);
        if (mark) mark("fft_zy");
        launch_fft_conv(a, st);
        if (mark) mark("fft_x_conv");
        launch_fft_inverse(a, st);
        if (mark) mark("ifft_yz");
        return;
    }
    for (auto& g : groups_) {
        CUFFT_CHECK(cufftSetStream(g.fwd, st));
        CUFFT_CHECK(cufftSetStream(g.inv, st));
    }
    for (auto& g : groups_)
        CUFFT_CHECK(cufftExecR2C(g.fwd, a.qreal + g.real_off, (cufftComplex*)(a.qcplx + g.cplx_off)));
    if (mark) mark("fft_r2c");
    launch_conv(a, st);
    if (mark) mark("conv");
    for (auto& g : groups_)
        CUFFT_CHECK(cufftExecC2R(g.inv, (cufftComplex*)(a.qcplx + g.cplx_off), a.qreal + g.real_off));
    if (mark) mark("fft_c2r");
}

bool Engine::check_status_and_grow() {
    const Status& s = *h_status_;
    last_tiles_ = s.tile_count;
    last_max_row_ = s.max_row;
    const int overflow = s.overflow | s.sticky;
    if (!overflow) return false;
    if (overflow & 2) {
        int want = (int)(s.max_row * 1.25) + 8;
        if (want > 2040) throw Error(6, "A tile row exceeds 2040 tiles: cutoff too large for the block layout");
        row_cap_ = std::max(row_cap_, want);
    }
    if (overflow & 1) tile_cap_ = (int)(std::max(tile_cap_, s.tile_count) * 1.5) + 4096;
    alloc_device();
    return true;
}

void Engine::run(bool host_io, cudaStream_t user, const double* d_pos, const double* h_pos_pinned,
                 bool host_results) {
    CUDA_CHECK(cudaSetDevice(dev_));
    if (!layout_ready_) {
        build_layout();
        alloc_device();
    }
    for (int attempt = 0; attempt < 4; attempt++) {
        update_rep_table();
        update_influence(user ? user : s_main_);
        // the control word is read when the evaluation runs (it follows the
        // synchronisation that ends every evaluation of this path)
        h_ctl_[0] = (force_build_ || skin_ <= 0.0) ? 1 : 0;
        force_build_ = false;
        cudaStream_t st = user ? user : s_main_;
        if (d_pos && d_pos != h_io_[0])  // (positions the graph reads in place need no copy)
            CUDA_CHECK(cudaMemcpyAsync((void*)A_.pos_in, d_pos, sizeof(double) * 3 * (size_t)n_in_,
                                       cudaMemcpyDeviceToDevice, st));
        if (h_pos_pinned)
            CUDA_CHECK(cudaMemcpyAsync((void*)A_.pos_in, h_pos_pinned, sizeof(double) * 3 * (size_t)n_in_,
                                       cudaMemcpyHostToDevice, st));
        if (profiling_) {
            // eager launches bracketed by events, one stream, for per-kernel timings
            times_.clear();
            std::vector<cudaEvent_t> ev;
            auto mark = [&](const char* name) {
                cudaEvent_t e;
                CUDA_CHECK(cudaEventCreate(&e));
                CUDA_CHECK(cudaEventRecord(e, st));
                ev.push_back(e);
                times_.push_back({name, 0.0});
            };
            const Args& a = A_;
            if (host_io)
                CUDA_CHECK(cudaMemcpyAsync((void*)a.pos_in, h_pos_, sizeof(double) * 3 * (size_t)n_in_,
                                           cudaMemcpyHostToDevice, st));
            CUDA_CHECK(cudaMemcpyAsync(d_params_, h_params_, param_bytes_, cudaMemcpyHostToDevice, st));
            CUDA_CHECK(cudaMemsetAsync(a.rep_hmax, 0, sizeof(unsigned) * (size_t)R_, st));
            mark("start");
            launch_prepare(a, st);
            launch_decide(a, st);
            mark("prepare");
            if (a.fused) {
                launch_find_tiles(a, st);
                mark("find_tiles");
            } else {
                launch_find(a, st);
                mark("find");
                launch_tiles(a, tile_grid_, st);
                mark("tiles");
            }
            launch_exceptions(a, st);
            mark("exceptions");
            if (method_ == NonbondedForce::PME) {
                launch_spread(a, st);
                mark("spread");
                pme_transforms(st, mark);
                launch_gather(a, st);
                mark("gather");
            }
            launch_finalize(a, st);
            mark("finalize");
            launch_output(a, st);
            mark("output");
            launch_matrix(a, st);
            mark("matrix");
            if (host_io) {
                CUDA_CHECK(cudaMemcpyAsync(h_results_, a.results, sizeof(double) * NUM_RES * (size_t)R_,
                                           cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaMemcpyAsync(h_forces_, a.f_out, sizeof(double) * 3 * (size_t)n_in_,
                                           cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaMemcpyAsync(h_fnb_, a.f_nb, sizeof(double) * 3 * (size_t)n_in_,
                                           cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaMemcpyAsync(h_matrix_, a.matrix, sizeof(double) * (size_t)R_ * R_,
                                           cudaMemcpyDeviceToHost, st));
            }
            CUDA_CHECK(cudaMemcpyAsync(h_status_, a.status, sizeof(Status), cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
            for (size_t k = 1; k < ev.size(); k++) {
                float ms = 0;
                CUDA_CHECK(cudaEventElapsedTime(&ms, ev[k - 1], ev[k]));
                times_[k].ms = ms;
            }
            for (auto e : ev) cudaEventDestroy(e);
            times_.erase(times_.begin());
        } else {
            const int mode = host_io ? 1 : ((h_pos_pinned || host_results) ? 2 : 0);
            cudaGraphExec_t& gx = mode == 1 ? graph_host_ : (mode == 2 ? graph_res_ : graph_dev_);
            if (!gx) {
                cudaGraph_t g;
                CUDA_CHECK(cudaStreamBeginCapture(s_main_, cudaStreamCaptureModeThreadLocal));
                try {
                    record(s_main_, mode);
                } catch (...) {
                    cudaStreamEndCapture(s_main_, &g);
                    throw;
                }
                CUDA_CHECK(cudaStreamEndCapture(s_main_, &g));
                CUDA_CHECK(cudaGraphInstantiate(&gx, g, 0));
                CUDA_CHECK(cudaGraphDestroy(g));
            }
            CUDA_CHECK(cudaGraphLaunch(gx, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
        }
        if (!check_status_and_grow()) {
            // the evaluation has run: later ones (launch_device) leave the build
            // to the device unless there is no skin
            h_ctl_[0] = skin_ <= 0.0 ? 1 : 0;
            return;
        }
    }
    throw Error(6, "Tile list capacity could not be established");
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister) can be the source or
// target of an asynchronous copy without a staging copy.
static bool is_pinned(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// The device address of a page-locked, mapped host buffer (cudaHostAlloc, or
// cudaHostRegister with mapping), which kernels can write over the host link; null
// for other memory.
static double* host_mapped(double* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || at.devicePointer == nullptr) return nullptr;
    return static_cast<double*>(at.devicePointer);
}

// Host copy split over a few threads (a single core moves ~10-20 GB/s).
static void par_memcpy(void* dst, const void* src, size_t bytes) {
    const size_t kMin = size_t(4) << 20;
    int nt = (int)std::min<size_t>(8, std::max<size_t>(1, bytes / kMin));
    if (nt <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    std::vector<std::thread> th;
    size_t chunk = (bytes + nt - 1) / nt;
    for (int t = 0; t < nt; t++) {
        size_t b = (size_t)t * chunk, e = std::min(bytes, b + chunk);
        if (b < e) th.emplace_back([=] { std::memcpy((char*)dst + b, (const char*)src + b, e - b); });
    }
    for (auto& x : th) x.join();
}

void Engine::evaluate(double* energies, double* forces, double* forces_nb, double* results, double* matrix) {
    evaluate_host(nullptr, energies, forces, forces_nb, results, matrix);
}

void Engine::evaluate_host(const double* pos, double* energies, double* forces, double* forces_nb, double* results,
                           double* matrix) {
    CUDA_CHECK(cudaSetDevice(dev_));
    const size_t bytes = sizeof(double) * 3 * (size_t)n_in_;
    const bool pin_in = pos && is_pinned(pos);
    // the layout and the profiling path read the staging copy
    if (pos && (!pin_in || !layout_ready_ || profiling_)) par_memcpy(h_pos_, pos, bytes);
    if (profiling_) {
        run(true, nullptr, nullptr);
    } else {
        // positions straight from a pinned caller buffer, else from the pinned
        // staging copy; forces written by the output kernel straight into a
        // page-locked caller buffer over the host link (no copy after the graph)
        double* zc = forces ? host_mapped(forces) : nullptr;
        h_io_[1] = zc;
        try {
            run(false, s_main_, nullptr, pin_in ? pos : h_pos_);
        } catch (...) {
            h_io_[1] = nullptr;
            throw;
        }
        h_io_[1] = nullptr;  // (the graph that read it has finished)
        const bool copy_f = forces && !zc;
        if (copy_f || forces_nb) {
            const bool pin_out = copy_f && is_pinned(forces);
            cudaStream_t st = s_main_;
            if (copy_f)
                CUDA_CHECK(cudaMemcpyAsync(pin_out ? forces : h_forces_, A_.f_out, bytes, cudaMemcpyDeviceToHost, st));
            if (forces_nb) CUDA_CHECK(cudaMemcpyAsync(h_fnb_, A_.f_nb, bytes, cudaMemcpyDeviceToHost, st));
            CUDA_CHECK(cudaStreamSynchronize(st));
            if (copy_f && !pin_out) par_memcpy(forces, h_forces_, bytes);
            if (forces_nb) par_memcpy(forces_nb, h_fnb_, bytes);
        }
        forces = nullptr;
        forces_nb = nullptr;
    }
    for (int r = 0; r < R_; r++) {
        if (energies) energies[r] = h_results_[(size_t)r * NUM_RES + RES_ENERGY];
    }
    if (forces) std::memcpy(forces, h_forces_, bytes);
    if (forces_nb) std::memcpy(forces_nb, h_fnb_, bytes);
    if (results) std::memcpy(results, h_results_, sizeof(double) * NUM_RES * (size_t)R_);
    if (matrix) std::memcpy(matrix, h_matrix_, sizeof(double) * (size_t)R_ * R_);
}

void Engine::run_device(const double* d_pos, cudaStream_t stream) {
    CUDA_CHECK(cudaSetDevice(dev_));
    if (!layout_ready_) {
        // the layout is built from positions: take them to the host once
        CUDA_CHECK(cudaMemcpyAsync(h_pos_, d_pos, sizeof(double) * 3 * (size_t)n_in_, cudaMemcpyDeviceToHost, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
        build_layout();
        alloc_device();
    }
    run(false, stream, d_pos);
}

void Engine::launch_device(const double* d_pos, cudaStream_t stream) {
    CUDA_CHECK(cudaSetDevice(dev_));
    if (!layout_ready_ || force_build_ || !graph_dev_) {
        // a new layout, new buffers or a forced build: the synchronous path (it
        // also establishes the capacities)
        run_device(d_pos, stream);
        return;
    }
    update_rep_table();
    if (!graph_dev_) {  // the box changed between orthorhombic and triclinic
        run_device(d_pos, stream);
        return;
    }
    update_influence(stream);
    // the control word stays as the last synchronous evaluation left it: 0 with a
    // skin (the device decides), 1 without one (every evaluation builds)
    if (d_pos != h_io_[0])
        CUDA_CHECK(cudaMemcpyAsync((void*)A_.pos_in, d_pos, sizeof(double) * 3 * (size_t)n_in_,
                                   cudaMemcpyDeviceToDevice, stream));
    CUDA_CHECK(cudaGraphLaunch(graph_dev_, stream));
}

void Engine::set_position_source(const double* d_pos) {
    CUDA_CHECK(cudaSetDevice(dev_));
    CUDA_CHECK(cudaDeviceSynchronize());  // no evaluation in flight reads the old one
    h_io_[0] = const_cast<double*>(d_pos);
}

bool Engine::poll_overflow() {
    // the status of the last evaluation (copied to the host at its end); sticky
    // carries the overflow of every build since the buffers were made
    if (!check_status_and_grow()) return false;
    return true;
}

void Engine::list_counts(long long* evals, long long* builds) const {
    long long c[2] = {0, 0};
    CUDA_CHECK(cudaSetDevice(dev_));
    CUDA_CHECK(cudaDeviceSynchronize());
    CUDA_CHECK(cudaMemcpy(c, d_counts_, sizeof(c), cudaMemcpyDeviceToHost));
    if (evals) *evals = c[0];
    if (builds) *builds = c[1];
}

void Engine::reorder_from_device(const double* d_pos, cudaStream_t stream) {
    CUDA_CHECK(cudaSetDevice(dev_));
    CUDA_CHECK(cudaMemcpyAsync(h_pos_, d_pos, sizeof(double) * 3 * (size_t)n_in_, cudaMemcpyDeviceToHost, stream));
    CUDA_CHECK(cudaStreamSynchronize(stream));
    layout_ready_ = false;
}

void Engine::evaluate_device(const double* d_pos, double* d_forces, double* d_results, cudaStream_t stream) {
    // the evaluation reads the caller's positions in place and writes the caller's
    // forces and result records itself (no copies before or after the graph); the
    // records and matrix also end in page-locked host memory
    double* const keep = h_io_[0];
    h_io_[0] = const_cast<double*>(d_pos);
    h_io_[1] = d_forces;
    h_io_[2] = d_results;
    try {
        if (!layout_ready_) {
            // the layout is built from positions: take them to the host once
            CUDA_CHECK(cudaMemcpyAsync(h_pos_, d_pos, sizeof(double) * 3 * (size_t)n_in_, cudaMemcpyDeviceToHost,
                                       stream));
            CUDA_CHECK(cudaStreamSynchronize(stream));
            build_layout();
            alloc_device();
        }
        run(false, stream, d_pos, nullptr, true);  // synchronises
    } catch (...) {
        h_io_[0] = keep;
        h_io_[1] = h_io_[2] = nullptr;
        throw;
    }
    h_io_[0] = keep;
    h_io_[1] = h_io_[2] = nullptr;
}

void Engine::reorder() { layout_ready_ = false; }

void Engine::set_nonbonded_params(int r, const double* q, const double* sig, const double* eps) {
    if (r < 0 || r >= R_) throw Error(2, "Replica index out of range");
    ReplicaSpec& s = specs_[r];
    std::memcpy(s.q.data(), q, sizeof(double) * (size_t)s.n);
    std::memcpy(s.sig.data(), sig, sizeof(double) * (size_t)s.n);
    std::memcpy(s.eps.data(), eps, sizeof(double) * (size_t)s.n);
    layout_ready_ = false;  // scaled charges, LJ pairs, exception charges and self energy follow
}

void Engine::backward(const double* d_g, double* d_dx, double* d_dd, double* d_dq, double* d_dsig, double* d_deps,
                      double* d_dpar, cudaStream_t stream) {
    CUDA_CHECK(cudaSetDevice(dev_));
    if (!layout_ready_) throw Error(3, "backward() needs a preceding evaluation");
    if (!adjoint_ && (d_dq || d_dsig || d_deps))
        throw Error(3, "Charge/sigma/epsilon gradients need a batch created with Adjoint=1");
    launch_adjoint(A_, d_g, d_dx, d_dd, d_dq, d_dsig, d_deps, d_dpar, stream);
    CUDA_CHECK(cudaGetLastError());
}

}  // namespace atm
