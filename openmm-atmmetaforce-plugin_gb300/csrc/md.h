// Langevin dynamics of R replicas driven by the batched ATM evaluation.
//
// The integrator is OpenMM's LangevinIntegrator (leapfrog form), the one the
// reference's test and examples step the ATM force with
// (python/tests/test_abfe.py:96-103, example/abfe/abfe.py:94-101):
//   v <- exp(-g dt) v + (1 - exp(-g dt))/g * f/m + sqrt(kT (1 - exp(-2 g dt)) / m) N(0,1)
//   x' <- x + dt v;  constrain x' (reference x);  v <- (x' - x)/dt;  x <- x'
// with f = ATM force (variable groups merged by the softplus weight) + group-0
// terms (bonds, angles, centroid and position restraints).  Forces are summed in
// 64-bit fixed point, the state is FP64, and the noise is Philox4x32-10 keyed by
// (seed, step, replica, atom), so a trajectory is reproducible bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace atm {

struct MdDev;  // kernel arguments (md.cu)

constexpr double kBoltz = 0.00831446261815324;  // kJ/mol/K (Avogadro x Boltzmann / 1000)

// Device records of the group-0 terms (user-order atom indices of the batch).
struct MdBond {
    int i, j, rep, pad;
    double length, k;
};
struct MdAngle {
    int i, j, l, rep;
    double angle, k;
};
struct MdPosRes {
    int p, rep, periodic, pad;
    double x0, y0, z0, fc, tol;
};
struct MdCentroid {
    int g1_off, g1_n, g2_off, g2_n, rep, pad;
    double kf, tol, off[3], m1, m2;
};
// A cluster of at most 4 atoms joined by at most 6 distance constraints (rigid
// water, X-H bonds), solved by SHAKE iterations in one thread.
constexpr int kConsAtoms = 4, kConsMax = 6;
struct MdConsGroup {
    int atom[kConsAtoms];  // batch indices, -1 unused
    int nc;
    int a[kConsMax], b[kConsMax];  // local atom slots of each constraint
    double d2[kConsMax];           // squared distances
};

// A rigid three-site water (O, H1, H2 with |O-H1| = |O-H2| and equal H masses),
// solved in closed form by SETTLE (Miyamoto and Kollman, J. Comput. Chem. 13,
// 952 (1992)): ra, rb, rc are the distances of the paper's canonical triangle
// (centre of mass to O, centre of mass to the H-H line, half the H-H distance).
struct MdSettle {
    int o, h1, h2, pad;
    double wo, wh;  // mass fractions of O and of each H
    double ra, rb, rc;
};

struct MdOptions {
    double temperature = 300.0;  // K
    double friction = 1.0;       // 1/ps
    double step_size = 0.002;    // ps
    uint64_t seed = 0;
    double constraint_tol = 1e-10;  // relative, on d^2
    int reorder_interval = 0;       // steps between re-sorts (0: when the tile count has grown by 20 %)
    double list_skin = 0.1;         // pair-list skin (nm, reduced to what the boxes allow); < 0: chosen
                                    // by autotune() at the first step
    int check_interval = 20;        // steps between host checks of the list capacities
    int fail_check = 0;             // test hook: the n-th list check reports an overflow (0: never)
};

class MDDriver {
public:
    MDDriver(const std::vector<const System*>& systems, int device, bool full_mode, const MdOptions& opt);
    ~MDDriver();
    MDDriver(const MDDriver&) = delete;
    MDDriver& operator=(const MDDriver&) = delete;

    Engine& engine() { return *eng_; }
    int replicas() const { return R_; }
    int total_atoms() const { return n_; }
    long long step_count() const { return step_; }

    void set_positions(const double* pos);  // host, 3n (batch order)
    void set_velocities(const double* vel);
    void set_velocities_to_temperature(double T, uint64_t seed);
    void set_param(int r, int which, double v);
    void set_integrator(double T, double friction, double dt);
    // Steps are enqueued without a host synchronisation per step: every
    // check_interval steps (and at the end of the call) the host reads the list
    // status; if a list build overflowed its capacity, the capacities grow, the
    // state goes back to the snapshot taken at the previous check and those steps
    // run again (the thermostat noise is a function of the step, so the redone
    // steps are the steps that should have run).
    void step(int nsteps);
    // Times the evaluation's launch space (Engine::autotune) and then `trials`
    // steps at each candidate pair-list skin (0 to 0.2 nm), keeps the fastest and
    // returns the report.  The state (positions, velocities, step count,
    // recording) is restored afterwards.  Needs positions and velocities.
    std::string autotune(int trials);
    // host outputs, nullable: positions, velocities, total forces (3n each);
    // per replica potential (group 0 + ATM) and kinetic energies; R x NUM_RES
    // results of the ATM evaluation at the current positions
    void get_state(double* pos, double* vel, double* forces, double* potential, double* kinetic, double* results);
    int reorders() const { return reorders_; }
    int redos() const { return redos_; }  // checks that sent the state back to a snapshot
    // Records of the ATM results (R x NUM_RES) and the R x R reduced-energy matrix
    // (beta = 1/kT of the integrator) every `interval` steps, at the positions the
    // step starts from, kept on the device in a ring of `capacity` records
    // (interval 0: off).  get_records copies the kept records, oldest first, and
    // empties the ring; outputs nullable, each sized for `max` records.
    void set_recording(int interval, int capacity);
    int get_records(long long* steps, double* results, double* matrices, int max);
    int constraint_groups() const { return n_cons_; }
    int settle_waters() const { return n_settle_; }

    const std::vector<int>& degrees_of_freedom() const { return dof_; }

private:
    void compute_forces(bool sync);
    void snapshot();
    void restore();
    bool check_lists();  // synchronises; true if steps since the snapshot must be redone
    void upload_terms(const std::vector<const System*>& systems);
    MdDev dev_args() const;

    std::unique_ptr<Engine> eng_;
    MdOptions opt_;
    int R_ = 0, n_ = 0, dev_ = 0;
    long long step_ = 0;
    bool forces_valid_ = false;
    bool have_positions_ = false;
    int reorders_ = 0;
    int base_tiles_ = 0;       // pair tiles after the last re-sort (at list skin base_skin_)
    double base_skin_ = -1.0;
    long long last_reorder_step_ = 0;
    std::vector<int> in_off_;
    std::vector<int> dof_;  // per replica: 3 x moving atoms - constraints

    cudaStream_t s_ = nullptr;
    cudaStream_t s_terms_ = nullptr;  // group-0 terms, beside the ATM evaluation
    cudaEvent_t ev_x_ = nullptr, ev_terms_ = nullptr;
    std::vector<void*> allocs_;
    double *x_ = nullptr, *v_ = nullptr, *xn_ = nullptr, *inv_m_ = nullptr, *sqrt_inv_m_ = nullptr;
    int* rep_of_ = nullptr;
    unsigned long long* fb_ = nullptr;  // group-0 forces, 3n fixed point
    double* e_terms_ = nullptr;         // one energy per term
    int* status_ = nullptr;             // SHAKE iterations exhausted (count)
    MdBond* bonds_ = nullptr;
    MdAngle* angles_ = nullptr;
    MdPosRes* posres_ = nullptr;
    MdCentroid* cent_ = nullptr;
    int* cent_idx_ = nullptr;
    double* cent_w_ = nullptr;
    MdConsGroup* cons_ = nullptr;
    MdSettle* settle_ = nullptr;
    int* free_ = nullptr;      // atoms in no constraint unit
    double* box_d_ = nullptr;  // 3 per replica
    int* rep_off_d_ = nullptr; // R + 1
    double* ke_d_ = nullptr;   // R
    double *x_snap_ = nullptr, *v_snap_ = nullptr;  // state at the last list check
    long long step_snap_ = 0, rec_count_snap_ = 0, rec_last_snap_ = -1;
    int checks_ = 0, redos_ = 0;
    bool tuned_ = false;
    int n_bonds_ = 0, n_angles_ = 0, n_posres_ = 0, n_cent_ = 0, n_cons_ = 0, n_settle_ = 0, n_free_ = 0;
    std::vector<int> term_rep_;  // replica of each term, in e_terms_ order
    // recording
    int rec_interval_ = 0, rec_cap_ = 0;
    long long rec_count_ = 0, rec_last_step_ = -1;
    std::vector<long long> rec_steps_;  // ring of step numbers
    double* rec_res_ = nullptr;         // rec_cap_ x R x NUM_RES
    double* rec_mat_ = nullptr;         // rec_cap_ x R x R
    void record_step();
    void update_beta();
};

}  // namespace atm
