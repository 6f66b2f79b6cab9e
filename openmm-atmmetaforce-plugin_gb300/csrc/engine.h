// GPU evaluation engine for R replicas of the ATM path (one CUDA graph per
// evaluation).  A single context is an engine with R = 1.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <functional>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "model.h"

namespace atm {

// Everything one replica contributes, copied out of its System.
struct ReplicaSpec {
    int n = 0;
    std::vector<double> q, sig, eps;
    std::vector<Exception> exc;
    std::vector<double> displ;  // 3n
    int method = 0;
    double cutoff = 1.0, epsRF = 78.3, alpha = 0.0;
    int grid[3] = {0, 0, 0};
    bool dispersion = false;
    double box[3] = {0, 0, 0};
    double tilt[3] = {0, 0, 0};  // b_x, c_x, c_y (OpenMM's reduced triclinic box vectors)
    double params[NUM_GLOBALS] = {0};
    bool var_nb = true;
};

// Build a ReplicaSpec from a System holding one NonbondedForce and one
// ATMMetaForce (the inner-system copy of ATMMetaForceImpl.cpp:32-67).
ReplicaSpec spec_from_system(const System& sys);

struct KernelTime {
    std::string name;
    double ms;
};

class Engine {
public:
    // adjoint: also accumulate the derivatives needed by backward() (difference mode only)
    Engine(std::vector<ReplicaSpec> reps, int device, bool full_mode, bool adjoint = false);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    int replicas() const { return R_; }
    int atoms(int r) const { return specs_[r].n; }
    int in_offset(int r) const { return in_off_[r]; }
    int total_atoms() const { return n_in_; }
    bool full_mode() const { return full_; }

    void set_positions(int r, const double* pos);
    void set_all_positions(const double* pos);
    void set_box(int r, const double* box, const double* tilt = nullptr);
    void set_param(int r, int which, double v);
    double param(int r, int which) const { return specs_[r].params[which]; }
    void set_displacements(int r, const double* displ);  // 3n, particle count unchanged
    void set_beta(double beta) { beta_ = beta; }
    // Neighbour-list skin (nm): lists are built at cutoff + skin and kept until an
    // atom has moved more than skin / 2 since their build (checked on the device at
    // every evaluation).  0 (the default): lists are built at every evaluation.
    void set_list_skin(double skin);
    // lists and pair tiles in one persistent kernel (k_find_tiles) or two kernels
    void set_fused(bool fused);
    // PME spreading by owner brick (each atom spread once, bricks added to int32
    // grids by atomics; used where the grids allow it) or by every brick a stencil
    // touches (each brick writes only its own points)
    void set_spread_owner(bool on);
    // the spreading brick edge (grid points; 0: spreading per atom with atomics into
    // the grids), as the autotuner would set it
    void set_spread_brick(int brick);
    // positions read in place by every evaluation from this device buffer (the MD
    // state), instead of copied into the engine's own; null: copied
    void set_position_source(const double* d_pos);
    void force_build() { force_build_ = true; }
    double list_skin() const { return skin_; }
    // evaluations run and how many of them built the lists (synchronises the device)
    void list_counts(long long* evals, long long* builds) const;

    // Host path: positions from the staging copy; outputs to host (nullable).
    void evaluate(double* energies, double* forces, double* forces_nb, double* results, double* matrix);
    // Host path with the caller's positions (nullable: the staging copy).  Page-locked
    // caller buffers are copied from / to directly; others go through pinned staging.
    void evaluate_host(const double* pos, double* energies, double* forces, double* forces_nb, double* results,
                       double* matrix);
    // Device path on the caller's stream.
    void evaluate_device(const double* d_pos, double* d_forces, double* d_results, cudaStream_t stream);
    // Device path without output copies: after it returns, forces_device() and
    // results_device() hold the evaluation at d_pos (valid until the next call).
    void run_device(const double* d_pos, cudaStream_t stream);
    // The same evaluation enqueued on the stream without waiting for it and
    // without reading its status: the caller synchronises the stream and calls
    // poll_overflow() before it trusts a result that a list build overflowed
    // (builds happen at the evaluations where atoms have moved beyond half the
    // skin, or when forced).
    void launch_device(const double* d_pos, cudaStream_t stream);
    // After a synchronisation of the stream of the evaluations: true if a list
    // build since the last poll overflowed its capacity (the capacities are then
    // grown and the next evaluation builds the lists again; the results of the
    // evaluations since that build are wrong and must be redone).
    bool poll_overflow();
    const double* forces_device() const { return A_.f_out; }
    const double* results_device() const { return A_.results; }
    const double* matrix_device() const { return A_.matrix; }
    const double* box(int r) const { return specs_[r].box; }
    const double* tilt(int r) const { return specs_[r].tilt; }
    // Re-sort from device positions at the next evaluation (the layout, tile
    // rows and exclusion masks are rebuilt; results do not change).
    void reorder_from_device(const double* d_pos, cudaStream_t stream);

    // Re-sort atoms from the current positions (exclusion masks follow).
    void reorder();

    // New charges, sigmas and epsilons of one replica's NonbondedForce (n each).
    void set_nonbonded_params(int r, const double* q, const double* sig, const double* eps);
    bool adjoint() const { return adjoint_; }
    // Gradients of sum_r g[r] W_r from the last evaluation (device pointers on
    // the given stream; outputs nullable, user order).
    void backward(const double* d_g, double* d_dx, double* d_dd, double* d_dq, double* d_dsig, double* d_deps,
                  double* d_dpar, cudaStream_t stream);

    // Times the evaluation over the tuning space (pair-tile CTAs per SM, PME
    // spreading brick size, PME stream overlap) and keeps the fastest; with
    // use_cache, a stored choice for the same GPU and workload is reused.
    // Returns a report.  Needs positions.
    std::string autotune(int trials, bool use_cache);
    void set_profiling(bool on) { profiling_ = on; }
    const std::vector<KernelTime>& kernel_times() const { return times_; }
    int launches_per_eval() const;
    int tile_dynamic() const;
    // tiles of the last evaluation, tile rows, and the largest row
    void stats(int* tiles, int* rows, int* max_row) const {
        if (tiles) *tiles = last_tiles_;
        if (rows) *rows = nrows_;
        if (max_row) *max_row = last_max_row_;
    }

private:
    void build_layout();
    void set_box_constants(RepDev& rd, const ReplicaSpec& s) const;
    static void recip_box(const ReplicaSpec& s, double* r);
    static double min_face_distance(const ReplicaSpec& s);
    float cutoff2() const;
    float list_cutoff2() const;
    void build_bricks();
    std::string tuning_key() const;
    void apply_tuning(int tile_per_sm, int brick, bool pme_stream, bool fused);
    bool load_tuning();
    void alloc_device();
    void free_device();
    void upload_static();
    void fill_args();
    void update_rep_table();
    // graph flavours: 0 device buffers only (MD, torch), 1 host staging copies of
    // positions, forces and results, 2 results and matrix to the host (positions
    // copied in before the launch, forces to a page-locked caller buffer or copied
    // after it)
    void record(cudaStream_t main, int mode);
    void pme_transforms(cudaStream_t st, const std::function<void(const char*)>& mark = nullptr);
    // host_results: the result records and matrix end in h_results_ / h_matrix_ (graph
    // flavour 2) without host positions
    void run(bool host_io, cudaStream_t user, const double* d_pos, const double* h_pos_pinned = nullptr,
             bool host_results = false);
    bool check_status_and_grow();
    void destroy_graphs();

    int R_ = 0, dev_ = 0;
    bool full_ = false;
    bool adjoint_ = false;
    std::vector<ReplicaSpec> specs_;
    std::vector<int> in_off_;
    int n_in_ = 0;
    int NA_ = 0, NB_ = 0, nrows_ = 0;
    int row_parts_ = 1;  // warps per tile-list row (1 unless rows are few)
    int row_cap_ = 192;
    int tile_cap_ = 0;
    int last_tiles_ = 0, last_max_row_ = 0;
    int method_ = 0;
    bool periodic_ = true;
    double cutoff_ = 1.0, alpha_ = 0.0, krf_ = 0.0, crf_ = 0.0;
    double beta_ = 1.0;
    double skin_ = 0.0;
    bool force_build_ = true;  // the next evaluation builds the lists
    long long* d_counts_ = nullptr;  // device: evaluations, list builds (kept across buffer rebuilds)
    bool layout_ready_ = false;
    bool profiling_ = false;
    int tile_grid_ = 0;
    int sms_ = 0, max_tile_per_sm_ = 1;
    int tune_tile_per_sm_ = 0;     // 0: as many as fit
    int tune_brick_ = 16;          // spreading brick edge (grid points)
    bool tune_pme_stream_ = true;  // PME on its own stream
    bool tune_fused_ = false;      // lists and pair tiles in one persistent kernel
    bool spread_owner_pref_ = true;  // spreading by owner brick where the grids allow it
    bool spread_owner_ = false;      // ... and in use (build_bricks)
    bool spread_atoms_ = false;      // spreading per atom (tune_brick_ 0, hand-written transform)

    // host copies of the layout
    std::vector<int> orig_, slot_of_, block_rep_, block_cls_;
    std::vector<float> qs_;
    std::vector<float2> lj_;
    std::vector<float4> displ_sorted_, block_d_;
    std::vector<int4> row_desc_;
    std::vector<int> ex_start_, dx_start_;
    std::vector<int2> ex_ent_, dx_ent_;
    std::vector<uint32_t> masks_;             // 32 x 32 exclusion masks (layout build)
    std::vector<uint32_t> masks16_;           // 16 x 16 sub-tile masks (device)
    std::vector<int> exs_start_, dxs_start_;  // per block: its exclusion sub-tiles
    std::vector<int4> exs_ent_, dxs_ent_;     //   (I16, J16, mask16 id, 0)
    std::vector<int4> exc_ij_;
    std::vector<ExcParam> exc_p_;
    std::vector<int> exc_cta_first_;
    std::vector<int> conv_cta_rep_;
    std::vector<long long> conv_cta_first_;
    std::vector<int> brick_cta_rep_;
    int brick_smem_ = 0;
    std::vector<float> moduli_;
    std::vector<RepDev> rep_host_;
    long long n_real_ = 0, n_cplx_ = 0;
    struct FftGroup {
        int K[3];
        int first_rep, count;
        cufftHandle fwd = 0, inv = 0;
        long long real_off, cplx_off;
    };
    std::vector<FftGroup> groups_;
    // hand-written transforms: used when every grid plane fits in shared memory
    bool use_fft_ = false;
    std::vector<float2> fft_tw_;
    std::vector<FftStage> fft_stages_;
    std::vector<int2> fft_plane_;
    std::vector<int4> fft_conv_;
    int fft_plane_smem_ = 0, fft_conv_smem_ = 0;
    bool infl_dirty_ = true;  // the influence-function table needs computing (new buffers or boxes)
    void update_influence(cudaStream_t st);

    // pinned host staging
    double* h_pos_ = nullptr;      // 3*n_in
    double* h_forces_ = nullptr;   // 3*n_in
    double* h_fnb_ = nullptr;      // 3*n_in
    double* h_results_ = nullptr;  // R*NUM_RES
    double* h_matrix_ = nullptr;   // R*R
    // The per-evaluation parameters in one page-locked block (list control word,
    // caller buffers, beta, replica table), which every evaluation copies to its
    // device mirror with one transfer; the four pointers below point into it.
    static constexpr size_t kParamReps = 64;  // byte offset of the replica table
    size_t param_bytes_ = 0;
    char* h_params_ = nullptr;
    char* d_params_ = nullptr;
    RepDev* h_reps_ = nullptr;     // R
    double* h_beta_ = nullptr;
    int* h_ctl_ = nullptr;         // list control word, copied to the device by every evaluation
    double** h_io_ = nullptr;      // caller buffers of the next evaluations (Args::io), copied to the
                                   // device by every evaluation: positions, forces, result records
    Status* h_status_ = nullptr;

    // device buffers
    Args A_{};
    void* d_mem_ = nullptr;
    std::vector<void*> d_allocs_;

    cudaStream_t s_main_ = nullptr, s_pme_ = nullptr;
    cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr, ev_fork2_ = nullptr, ev_join2_ = nullptr;
    cudaGraphExec_t graph_host_ = nullptr, graph_dev_ = nullptr, graph_res_ = nullptr;
    std::vector<KernelTime> times_;
};

}  // namespace atm
