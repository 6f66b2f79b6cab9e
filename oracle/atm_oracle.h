/*
 * atm_oracle.h -- FP64 CPU restatement of the ATMMetaForce evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path and
 * the timed CPU baseline; the product library never links it and never calls it.
 *
 * What it restates (reference paths are relative to the reference project):
 *   - the ATM merge: SoftCoreF, softplus W(u), dW/du and the force
 *     hybridisation of platforms/reference/src/ReferenceATMMetaForceKernels.cpp:26-113;
 *   - the coordinate displacement of the second state
 *     (ReferenceATMMetaForceKernels.cpp:116-124);
 *   - the inner NonbondedForce evaluation that ATMMetaForceImpl.cpp:113,116 delegates
 *     to OpenMM: Lennard-Jones with Lorentz-Berthelot combination and a plain
 *     cutoff, Coulomb as plain (NoCutoff), reaction field (cutoff methods) or
 *     smooth PME (Essmann et al., J. Chem. Phys. 103, 8577 (1995)) with
 *     exclusions and exceptions, following the NonbondedForce definitions in
 *     OpenMM's user guide (theory chapter).
 *
 * Units: nm, kJ/mol, elementary charges.  Periodic boxes are OpenMM's reduced
 * triclinic form a = (box[0], 0, 0), b = (tilt[0], box[1], 0), c = (tilt[1],
 * tilt[2], box[2]) (orthorhombic when the tilts are zero), with OpenMM's minimum
 * image: subtract c, then b, then a, each rounded to the nearest multiple.
 */
#ifndef ATM_ORACLE_H
#define ATM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Nonbonded methods, numbered like OpenMM's NonbondedForce::NonbondedMethod. */
#define ONB_NOCUTOFF 0
#define ONB_CUTOFF_NONPERIODIC 1
#define ONB_CUTOFF_PERIODIC 2
#define ONB_PME 4

/* Coulomb constant 1/(4 pi eps0) in kJ mol^-1 nm e^-2 (OpenMM 7.x value). */
#define ONB_ONE_4PI_EPS0 138.935456

typedef struct {
    int n;                                   /* particles */
    const double *charge, *sigma, *epsilon;  /* per particle */
    int n_exc;                               /* exceptions (excluded pairs included) */
    const int *exc_i, *exc_j;
    const double *exc_qq, *exc_sig, *exc_eps;
    int method;                              /* ONB_* */
    double cutoff;                           /* nm */
    double eps_rf;                           /* reaction-field dielectric */
    double alpha;                            /* Ewald splitting parameter, nm^-1 */
    int grid[3];                             /* PME grid */
    int order;                               /* PME B-spline order */
    int use_disp_corr;                       /* long-range LJ correction */
    double box[3];                           /* diagonal of the box vectors, nm */
    double tilt[3];                          /* b_x, c_x, c_y of the box vectors, nm */
} onb_t;

typedef struct {
    double direct;      /* pair terms within the cutoff */
    double exceptions;  /* exception pairs (1-4 etc.) and, under PME, exclusion corrections */
    double recip;       /* PME reciprocal-space energy */
    double self;        /* PME self energy */
    double disp;        /* dispersion correction */
} oterms_t;

/* Number of OpenMP threads used by the evaluators (1 = deterministic serial path). */
int o_set_threads(int n);

/* Energy and forces of the NonbondedForce at positions pos[n*3].
 * pos_cut (nullable) decides which pairs fall inside the cutoff; it is how finite
 * differences freeze the pair set.  forces (nullable) is overwritten. */
int onb_energy_forces(const onb_t* s, const double* pos, const double* pos_cut,
                      double* energy, double* forces, oterms_t* terms);

/* Derivatives of the energy with respect to each particle's charge, sigma and
 * epsilon (any pointer may be NULL).  pos_cut as above. */
int onb_param_derivs(const onb_t* s, const double* pos, const double* pos_cut,
                     double* dUdq, double* dUdsig, double* dUdeps);

/* Exact Ewald reciprocal sum over |m| <= kmax in each direction; for checking PME. */
int onb_ewald_recip_exact(const onb_t* s, const double* pos, int kmax, double* energy, double* forces);

/* Soft-core map of ReferenceATMMetaForceKernels.cpp:26-37. */
double o_softcore(double u, double umax, double a, double ub, double* fp);

/* The ATM merge of ReferenceATMMetaForceKernels.cpp:56-113.
 * params = {lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction}.
 * out = {energy, perturbation energy usc, sp = dW/du, W, u_raw, e0, bfp, fp}.
 * f_out[n*3] (nullable) receives the hybrid force dir>0: sp*F2+(1-sp)*F1,
 * dir<=0: sp*F1+(1-sp)*F2. */
void o_atm_merge(double E1, double E2, const double* params, int n,
                 const double* F1, const double* F2, double* f_out, double* out);

/* Derivatives of W with respect to {lambda1, lambda2, alpha, u0, w0} at a given
 * soft-cored perturbation energy usc (closed form of the softplus in
 * ReferenceATMMetaForceKernels.cpp:89-95). */
void o_softplus_param_grad(double usc, const double* params, double* dW);

/* Full ATM evaluation: state 1 at pos, state 2 at pos+displ, then the merge.
 * forces[n*3] (nullable) receives the ATM force; out as in o_atm_merge;
 * E12 (nullable) receives {E1, E2}; F12 (nullable, 2*n*3) receives F1 then F2. */
int o_atm_eval(const onb_t* s, const double* pos, const double* displ, const double* params,
               const double* pos_cut, double* forces, double* out, double* E12, double* F12);

/* PME grid rule of OpenMM's NonbondedForce documentation:
 * alpha = sqrt(-ln(2 tol))/rc, n_d = ceil(2 alpha L_d / (3 tol^(1/5))), at least 6.
 * legal != 0 rounds each n_d up to a size whose only prime factors are 2,3,5,7. */
void o_pme_parameters(double cutoff, double tol, const double* box, int legal,
                      double* alpha, int* grid);

/* In-place 3D complex FFT on a row-major (z fastest) grid of interleaved
 * re/im doubles; sign = -1 forward, +1 backward, unnormalised. */
int o_fft3d(double* data, const int* dims, int sign);

#ifdef __cplusplus
}
#endif
#endif
