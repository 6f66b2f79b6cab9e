/*
 * atm_oracle.c -- FP64 CPU restatement of the ATMMetaForce evaluation path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product links or calls this file.
 *
 * The reference plugin delegates the two inner energy evaluations to OpenMM
 * (openmmapi/src/ATMMetaForceImpl.cpp:113,116) and merges them on the host
 * (platforms/reference/src/ReferenceATMMetaForceKernels.cpp:56-113).  This file
 * restates both halves in double precision:
 *   - nonbonded energy/forces with OpenMM NonbondedForce semantics (documented
 *     in OpenMM's user guide): LJ with Lorentz-Berthelot rules and a plain
 *     cutoff; Coulomb plain (NoCutoff), reaction field (cutoff methods) or
 *     smooth PME (Essmann et al. 1995, order-n cardinal B-splines); exceptions
 *     replace the pair interaction; under PME every exception pair also gets the
 *     -q_i q_j erf(alpha r)/r correction for the reciprocal sum;
 *   - the soft-core / softplus merge, line for line in meaning with the
 *     reference's Reference platform.
 *
 * Parity pin: the TEMOA-G1 ABFE perturbation energy of the reference's own test
 * (python/tests/test_abfe.py:148,150, u = 58.2 +- 0.1 kJ/mol) is recomputed by
 * this oracle in tests/test_oracle_pin.py from a fixture generated out of the
 * reference's test inputs.
 */
#include "atm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int g_threads = 1;

int o_set_threads(int n) {
    g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
    return g_threads;
#else
    g_threads = 1;
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Small helpers                                                               */
/* ------------------------------------------------------------------------- */

static inline double min_image(double d, double L) { return d - L * floor(d / L + 0.5); }

static int is_periodic(int method) { return method == ONB_CUTOFF_PERIODIC || method == ONB_PME; }

static int is_triclinic(const onb_t* s) { return s->tilt[0] != 0.0 || s->tilt[1] != 0.0 || s->tilt[2] != 0.0; }

/* The periodic shift that takes d to its minimum image (OpenMM's reduced-box
 * rule: c, then b, then a), returned in shift (d - shift is the image). */
static void image_shift(const onb_t* s, const double* d, double* shift) {
    double v[3] = {d[0], d[1], d[2]};
    double k = floor(v[2] / s->box[2] + 0.5);
    v[0] -= k * s->tilt[1];
    v[1] -= k * s->tilt[2];
    v[2] -= k * s->box[2];
    k = floor(v[1] / s->box[1] + 0.5);
    v[0] -= k * s->tilt[0];
    v[1] -= k * s->box[1];
    k = floor(v[0] / s->box[0] + 0.5);
    v[0] -= k * s->box[0];
    for (int a = 0; a < 3; a++) shift[a] = d[a] - v[a];
}

/* Reciprocal box (rows r_i, as OpenMM's recipBoxVectors): the fractional
 * coordinate along box vector d of position p is sum_i p_i r[i][d]. */
static void recip_box(const onb_t* s, double r[3][3]) {
    const double ax = s->box[0], by = s->box[1], cz = s->box[2];
    const double bx = s->tilt[0], cx = s->tilt[1], cy = s->tilt[2];
    memset(r, 0, 9 * sizeof(double));
    r[0][0] = 1.0 / ax;
    r[1][0] = -bx / (ax * by);
    r[1][1] = 1.0 / by;
    r[2][0] = (bx * cy - by * cx) / (ax * by * cz);
    r[2][1] = -cy / (by * cz);
    r[2][2] = 1.0 / cz;
}

/* Sorted CSR adjacency of exception partners, for the "is this pair an
 * exception" test of the pair loop. */
typedef struct {
    int* start;
    int* list;
} excl_csr;

static int cmp_int(const void* a, const void* b) {
    int x = *(const int*)a, y = *(const int*)b;
    return (x > y) - (x < y);
}

static int build_excl(const onb_t* s, excl_csr* e) {
    e->start = (int*)calloc((size_t)s->n + 1, sizeof(int));
    e->list = (int*)malloc(sizeof(int) * (size_t)(2 * s->n_exc + 1));
    if (!e->start || !e->list) return -1;
    for (int k = 0; k < s->n_exc; k++) {
        e->start[s->exc_i[k] + 1]++;
        e->start[s->exc_j[k] + 1]++;
    }
    for (int i = 0; i < s->n; i++) e->start[i + 1] += e->start[i];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(s->n + 1));
    memcpy(fill, e->start, sizeof(int) * (size_t)(s->n + 1));
    for (int k = 0; k < s->n_exc; k++) {
        e->list[fill[s->exc_i[k]]++] = s->exc_j[k];
        e->list[fill[s->exc_j[k]]++] = s->exc_i[k];
    }
    free(fill);
    for (int i = 0; i < s->n; i++)
        qsort(e->list + e->start[i], (size_t)(e->start[i + 1] - e->start[i]), sizeof(int), cmp_int);
    return 0;
}

static void free_excl(excl_csr* e) {
    free(e->start);
    free(e->list);
}

static int excluded(const excl_csr* e, int i, int j) {
    int lo = e->start[i], hi = e->start[i + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int v = e->list[mid];
        if (v == j) return 1;
        if (v < j) lo = mid + 1; else hi = mid - 1;
    }
    return 0;
}

/* One pair inside the cutoff.  Returns energy, and fr = -(dE/dr)/r so that the
 * force on j is fr*(r_j - r_i).  Derivative-with-respect-to-parameter outputs
 * (dq = dE/d(q_i q_j), ds = dE/d sigma_ij, de = dE/d eps_ij) are optional. */
static inline double pair_energy(const onb_t* s, double r2, double qq, double sig, double eps,
                                 double* fr, double* dqq, double* dsig, double* deps) {
    const double k = ONB_ONE_4PI_EPS0;
    double r = sqrt(r2), inv_r = 1.0 / r, inv_r2 = inv_r * inv_r;
    double e = 0.0, f = 0.0, dq = 0.0, ds = 0.0, de = 0.0;
    if (eps != 0.0) {
        double sr2 = sig * sig * inv_r2;
        double s6 = sr2 * sr2 * sr2;
        e += 4.0 * eps * (s6 * s6 - s6);
        f += 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6) * inv_r2;
        de = 4.0 * (s6 * s6 - s6);
        ds = 4.0 * eps * (12.0 * s6 * s6 - 6.0 * s6) / sig;
    }
    if (qq != 0.0 || dqq) {
        double phi, fphi;
        if (s->method == ONB_NOCUTOFF) {
            phi = inv_r;
            fphi = inv_r * inv_r2;
        } else if (s->method == ONB_PME) {
            double ar = s->alpha * r;
            double ec = erfc(ar);
            phi = ec * inv_r;
            fphi = (ec * inv_r + 2.0 * s->alpha / sqrt(M_PI) * exp(-ar * ar)) * inv_r2;
        } else {
            double rc = s->cutoff, er = s->eps_rf;
            double krf = (er - 1.0) / ((2.0 * er + 1.0) * rc * rc * rc);
            double crf = 3.0 * er / ((2.0 * er + 1.0) * rc);
            phi = inv_r + krf * r2 - crf;
            fphi = inv_r * inv_r2 - 2.0 * krf;
        }
        e += k * qq * phi;
        f += k * qq * fphi;
        dq = k * phi;
    }
    *fr = f;
    if (dqq) *dqq = dq;
    if (dsig) *dsig = ds;
    if (deps) *deps = de;
    return e;
}

/* ------------------------------------------------------------------------- */
/* Direct space                                                                */
/* ------------------------------------------------------------------------- */

typedef struct {
    const onb_t* s;
    const double* pos;
    const double* pc;   /* positions deciding the cutoff */
    const excl_csr* ex;
    double* forces;     /* may be NULL */
    double* dUdq;       /* may be NULL (parameter-derivative mode) */
    double* dUdsig;
    double* dUdeps;
    int tric;           /* triclinic box: images by the reduced-box rule */
} direct_job;

static inline double do_pair(const direct_job* J, int i, int j, double* fi_acc, double* fj_acc) {
    const onb_t* s = J->s;
    int per = is_periodic(s->method);
    double dc[3], d[3], r2c = 0.0, r2 = 0.0;
    for (int a = 0; a < 3; a++) {
        dc[a] = J->pc[3 * j + a] - J->pc[3 * i + a];
        d[a] = J->pos[3 * j + a] - J->pos[3 * i + a];
    }
    if (per && J->tric) {
        /* the same image shift is applied to the evaluation geometry */
        double shift[3];
        image_shift(s, dc, shift);
        for (int a = 0; a < 3; a++) {
            dc[a] -= shift[a];
            d[a] -= shift[a];
        }
    } else if (per) {
        /* orthorhombic: the axes are independent */
        for (int a = 0; a < 3; a++) {
            const double shift = s->box[a] * floor(dc[a] / s->box[a] + 0.5);
            dc[a] -= shift;
            d[a] -= shift;
        }
    }
    for (int a = 0; a < 3; a++) {
        r2c += dc[a] * dc[a];
        r2 += d[a] * d[a];
    }
    if (s->method != ONB_NOCUTOFF && r2c >= s->cutoff * s->cutoff) return 0.0;
    if (excluded(J->ex, i, j)) return 0.0;
    double sig = 0.5 * (s->sigma[i] + s->sigma[j]);
    double eps = sqrt(s->epsilon[i] * s->epsilon[j]);
    double qq = s->charge[i] * s->charge[j];
    double fr, dq, ds, de;
    int pd = J->dUdq || J->dUdsig || J->dUdeps;
    double e = pair_energy(s, r2, qq, sig, eps, &fr, pd ? &dq : NULL, pd ? &ds : NULL, pd ? &de : NULL);
    if (fi_acc) {
        for (int a = 0; a < 3; a++) {
            fi_acc[a] -= fr * d[a];
            fj_acc[a] += fr * d[a];
        }
    }
    if (pd) {
        /* dE/dq_i = dE/dqq * q_j; dE/dsig_i = dE/dsig_ij / 2;
           dE/deps_i = dE/deps_ij * eps_j / (2 eps_ij) */
        if (J->dUdq) {
            J->dUdq[i] += dq * s->charge[j];
            J->dUdq[j] += dq * s->charge[i];
        }
        if (J->dUdsig) {
            J->dUdsig[i] += 0.5 * ds;
            J->dUdsig[j] += 0.5 * ds;
        }
        if (J->dUdeps && eps > 0.0) {
            J->dUdeps[i] += de * s->epsilon[j] / (2.0 * eps);
            J->dUdeps[j] += de * s->epsilon[i] / (2.0 * eps);
        }
    }
    return e;
}

/* Pairs within the cutoff, found with a cell list on pos_cut when every
 * periodic dimension holds at least three cells, by all-pairs otherwise. */
static double direct_space(const direct_job* J) {
    const onb_t* s = J->s;
    int n = s->n;
    double energy = 0.0;
    int use_cells = is_periodic(s->method) && !is_triclinic(s);
    int nc[3] = {1, 1, 1};
    if (use_cells) {
        for (int a = 0; a < 3; a++) {
            nc[a] = (int)floor(s->box[a] / s->cutoff);
            if (nc[a] < 3) use_cells = 0;
        }
    }
    int nthreads = g_threads;
    int pd = J->dUdq || J->dUdsig || J->dUdeps;
    if (pd) nthreads = 1; /* parameter derivatives are a small-case checker */
    double* fbuf = NULL;
    if (J->forces) {
        fbuf = (double*)calloc((size_t)nthreads * 3 * (size_t)n, sizeof(double));
    }
    if (!use_cells) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16) reduction(+ : energy)
#endif
        for (int i = 0; i < n; i++) {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double* fb = fbuf ? fbuf + (size_t)t * 3 * n : NULL;
            for (int j = i + 1; j < n; j++)
                energy += do_pair(J, i, j, fb ? fb + 3 * i : NULL, fb ? fb + 3 * j : NULL);
        }
    } else {
        int ncell = nc[0] * nc[1] * nc[2];
        int* head = (int*)malloc(sizeof(int) * (size_t)ncell);
        int* next = (int*)malloc(sizeof(int) * (size_t)n);
        int* cell_of = (int*)malloc(sizeof(int) * (size_t)n);
        for (int c = 0; c < ncell; c++) head[c] = -1;
        for (int i = n - 1; i >= 0; i--) {
            int ci[3];
            for (int a = 0; a < 3; a++) {
                double x = J->pc[3 * i + a];
                x -= s->box[a] * floor(x / s->box[a]);
                int c = (int)floor(x / s->box[a] * nc[a]);
                if (c < 0) c = 0;
                if (c >= nc[a]) c = nc[a] - 1;
                ci[a] = c;
            }
            int c = (ci[0] * nc[1] + ci[1]) * nc[2] + ci[2];
            cell_of[i] = c;
            next[i] = head[c];
            head[c] = i;
        }
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4) reduction(+ : energy)
#endif
        for (int c = 0; c < ncell; c++) {
            int t = 0;
#ifdef _OPENMP
            t = omp_get_thread_num();
#endif
            double* fb = fbuf ? fbuf + (size_t)t * 3 * n : NULL;
            int cx = c / (nc[1] * nc[2]), cy = (c / nc[2]) % nc[1], cz = c % nc[2];
            for (int i = head[c]; i >= 0; i = next[i]) {
                for (int ox = -1; ox <= 1; ox++)
                    for (int oy = -1; oy <= 1; oy++)
                        for (int oz = -1; oz <= 1; oz++) {
                            int nx = (cx + ox + nc[0]) % nc[0];
                            int ny = (cy + oy + nc[1]) % nc[1];
                            int nz = (cz + oz + nc[2]) % nc[2];
                            int c2 = (nx * nc[1] + ny) * nc[2] + nz;
                            for (int j = head[c2]; j >= 0; j = next[j]) {
                                if (j <= i) continue;
                                energy += do_pair(J, i, j, fb ? fb + 3 * i : NULL, fb ? fb + 3 * j : NULL);
                            }
                        }
            }
        }
        free(head);
        free(next);
        free(cell_of);
    }
    if (fbuf) {
        for (int t = 0; t < nthreads; t++)
            for (int k = 0; k < 3 * n; k++) J->forces[k] += fbuf[(size_t)t * 3 * n + k];
        free(fbuf);
    }
    return energy;
}

/* Exceptions: a nonzero exception is Coulomb chargeProd/r plus LJ(sigma, eps)
 * with no cutoff and no periodic image; under PME every exception pair also
 * subtracts the reciprocal-space interaction q_i q_j erf(alpha r)/r, computed
 * at the minimum-image separation. */
static double exceptions_term(const onb_t* s, const double* pos, double* forces, double* dUdq,
                              double* dUdsig, double* dUdeps) {
    const double k = ONB_ONE_4PI_EPS0;
    double energy = 0.0;
    (void)dUdsig;
    (void)dUdeps;
    for (int m = 0; m < s->n_exc; m++) {
        int i = s->exc_i[m], j = s->exc_j[m];
        double d[3], r2 = 0.0;
        for (int a = 0; a < 3; a++) {
            d[a] = pos[3 * j + a] - pos[3 * i + a];
            r2 += d[a] * d[a];
        }
        double fr = 0.0;
        if (s->exc_qq[m] != 0.0 || s->exc_eps[m] != 0.0) {
            double r = sqrt(r2), inv_r2 = 1.0 / r2;
            double e = k * s->exc_qq[m] / r;
            double f = k * s->exc_qq[m] / (r * r2);
            if (s->exc_eps[m] != 0.0) {
                double sr2 = s->exc_sig[m] * s->exc_sig[m] * inv_r2;
                double s6 = sr2 * sr2 * sr2;
                e += 4.0 * s->exc_eps[m] * (s6 * s6 - s6);
                f += 4.0 * s->exc_eps[m] * (12.0 * s6 * s6 - 6.0 * s6) * inv_r2;
            }
            energy += e;
            fr += f;
        }
        if (s->method == ONB_PME) {
            double dm[3], sh[3], r2m = 0.0;
            image_shift(s, d, sh);
            for (int a = 0; a < 3; a++) {
                dm[a] = d[a] - sh[a];
                r2m += dm[a] * dm[a];
            }
            double r = sqrt(r2m);
            double ar = s->alpha * r;
            double qq = s->charge[i] * s->charge[j];
            if (r > 0.0) {
                double ef = erf(ar);
                energy -= k * qq * ef / r;
                double fm = k * qq * (2.0 * s->alpha / sqrt(M_PI) * exp(-ar * ar) - ef / r) / r2m;
                if (forces) {
                    for (int a = 0; a < 3; a++) {
                        forces[3 * i + a] -= fm * dm[a];
                        forces[3 * j + a] += fm * dm[a];
                    }
                }
                if (dUdq) {
                    dUdq[i] -= k * s->charge[j] * ef / r;
                    dUdq[j] -= k * s->charge[i] * ef / r;
                }
            } else if (dUdq) {
                /* coincident pair: limit of erf(a r)/r */
                dUdq[i] -= k * s->charge[j] * 2.0 * s->alpha / sqrt(M_PI);
                dUdq[j] -= k * s->charge[i] * 2.0 * s->alpha / sqrt(M_PI);
            }
            if (r == 0.0) energy -= k * qq * 2.0 * s->alpha / sqrt(M_PI);
        }
        if (forces && fr != 0.0) {
            for (int a = 0; a < 3; a++) {
                forces[3 * i + a] -= fr * d[a];
                forces[3 * j + a] += fr * d[a];
            }
        }
    }
    return energy;
}

/* Long-range dispersion correction of NonbondedForce (OpenMM user guide):
 * E = 8 pi N^2 / V * (<eps sigma^12>/(9 rc^9) - <eps sigma^6>/(3 rc^3)), the
 * averages running over all particle pairs, self pairs included, grouped into
 * classes of identical (sigma, epsilon). */
static double dispersion_correction(const onb_t* s) {
    if (!s->use_disp_corr || !is_periodic(s->method)) return 0.0;
    int n = s->n;
    double* cs = (double*)malloc(sizeof(double) * (size_t)n);
    double* ce = (double*)malloc(sizeof(double) * (size_t)n);
    double* cnt = (double*)malloc(sizeof(double) * (size_t)n);
    int ncls = 0;
    for (int i = 0; i < n; i++) {
        int c;
        for (c = 0; c < ncls; c++)
            if (cs[c] == s->sigma[i] && ce[c] == s->epsilon[i]) break;
        if (c == ncls) {
            cs[c] = s->sigma[i];
            ce[c] = s->epsilon[i];
            cnt[c] = 0.0;
            ncls++;
        }
        cnt[c] += 1.0;
    }
    double sum1 = 0.0, sum2 = 0.0;
    for (int a = 0; a < ncls; a++)
        for (int b = a; b < ncls; b++) {
            double sig = 0.5 * (cs[a] + cs[b]);
            double eps = sqrt(ce[a] * ce[b]);
            double count = (a == b) ? cnt[a] * (cnt[a] + 1.0) / 2.0 : cnt[a] * cnt[b];
            double s6 = pow(sig, 6.0);
            sum1 += count * eps * s6 * s6;
            sum2 += count * eps * s6;
        }
    free(cs);
    free(ce);
    free(cnt);
    double N = (double)n;
    double npairs = N * (N + 1.0) / 2.0;
    sum1 /= npairs;
    sum2 /= npairs;
    double rc = s->cutoff;
    double vol = s->box[0] * s->box[1] * s->box[2];
    return 8.0 * M_PI * N * N * (sum1 / (9.0 * pow(rc, 9.0)) - sum2 / (3.0 * pow(rc, 3.0))) / vol;
}

/* ------------------------------------------------------------------------- */
/* Mixed-radix FFT (recursive Cooley-Tukey, in-place combine)                  */
/* ------------------------------------------------------------------------- */

static int smallest_factor(int n) {
    for (int p = 2; p * p <= n; p++)
        if (n % p == 0) return p;
    return n;
}

/* out[k] = sum_j in[j*is] w^(j k), w = tw[tstep] = exp(sign 2 pi i / n). */
static void fft_rec(const double* in, long is, double* out, int n, const double* tw, int N, int tstep,
                    double* tmp) {
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; r++) fft_rec(in + 2 * r * is, is * p, out + 2 * r * m, m, tw, N, tstep * p, tmp);
    for (int k = 0; k < m; k++) {
        for (int r = 0; r < p; r++) {
            tmp[2 * r] = out[2 * (r * m + k)];
            tmp[2 * r + 1] = out[2 * (r * m + k) + 1];
        }
        for (int q = 0; q < p; q++) {
            double ar = 0.0, ai = 0.0;
            int kk = k + q * m;
            for (int r = 0; r < p; r++) {
                long idx = ((long)r * kk) % n;
                double wr = tw[2 * idx * tstep], wi = tw[2 * idx * tstep + 1];
                ar += tmp[2 * r] * wr - tmp[2 * r + 1] * wi;
                ai += tmp[2 * r] * wi + tmp[2 * r + 1] * wr;
            }
            out[2 * kk] = ar;
            out[2 * kk + 1] = ai;
        }
    }
    (void)N;
}

int o_fft3d(double* data, const int* dims, int sign) {
    int maxd = dims[0];
    if (dims[1] > maxd) maxd = dims[1];
    if (dims[2] > maxd) maxd = dims[2];
    long strides[3] = {(long)dims[1] * dims[2], dims[2], 1};
    for (int ax = 0; ax < 3; ax++) {
        int n = dims[ax];
        double* tw = (double*)malloc(sizeof(double) * 2 * (size_t)n);
        for (int k = 0; k < n; k++) {
            double a = sign * 2.0 * M_PI * k / n;
            tw[2 * k] = cos(a);
            tw[2 * k + 1] = sin(a);
        }
        int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
        long nlines = (long)dims[o1] * dims[o2];
#ifdef _OPENMP
#pragma omp parallel num_threads(g_threads)
#endif
        {
            double* line = (double*)malloc(sizeof(double) * 2 * (size_t)n);
            double* out = (double*)malloc(sizeof(double) * 2 * (size_t)n);
            double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (long L = 0; L < nlines; L++) {
                long a1 = L / dims[o2], a2 = L % dims[o2];
                long base = a1 * strides[o1] + a2 * strides[o2];
                for (int k = 0; k < n; k++) {
                    line[2 * k] = data[2 * (base + k * strides[ax])];
                    line[2 * k + 1] = data[2 * (base + k * strides[ax]) + 1];
                }
                fft_rec(line, 1, out, n, tw, n, 1, tmp);
                for (int k = 0; k < n; k++) {
                    data[2 * (base + k * strides[ax])] = out[2 * k];
                    data[2 * (base + k * strides[ax]) + 1] = out[2 * k + 1];
                }
            }
            free(line);
            free(out);
            free(tmp);
        }
        free(tw);
    }
    (void)maxd;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Smooth PME                                                                  */
/* ------------------------------------------------------------------------- */

/* w[k] = M_n(t+k), dw[k] = M_n'(t+k) for k = 0..n-1, t in [0,1), from the
 * cardinal B-spline recursion M_m(x) = (x M_{m-1}(x) + (m-x) M_{m-1}(x-1))/(m-1). */
static void bspline(double t, int n, double* w, double* dw) {
    double a[16];
    for (int k = 0; k < n; k++) a[k] = 0.0;
    a[0] = t;
    a[1] = 1.0 - t;
    for (int m = 3; m <= n; m++) {
        if (m == n) {
            dw[0] = a[0];
            for (int k = 1; k < n; k++) dw[k] = a[k] - a[k - 1];
        }
        double b[16];
        for (int k = 0; k < m; k++) {
            double x = t + k;
            double cur = (k < m - 1) ? a[k] : 0.0;
            double prev = (k > 0) ? a[k - 1] : 0.0;
            b[k] = (x * cur + (m - x) * prev) / (m - 1);
        }
        for (int k = 0; k < m; k++) a[k] = b[k];
    }
    if (n == 2) {
        dw[0] = 1.0;
        dw[1] = -1.0;
    }
    for (int k = 0; k < n; k++) w[k] = a[k];
}

/* |sum_{k=0}^{n-2} M_n(k+1) e^{2 pi i m k / K}|^2, with the usual repair of
 * vanishing values by the mean of the neighbours. */
static void bspline_moduli(int K, int order, double* mod) {
    double w[16], dw[16];
    bspline(0.0, order, w, dw); /* w[k] = M_n(k) */
    double c[16];
    for (int k = 0; k < order; k++) c[k] = (k + 1 < order) ? w[k + 1] : 0.0;
    for (int m = 0; m < K; m++) {
        double sc = 0.0, ss = 0.0;
        for (int k = 0; k < order; k++) {
            double arg = 2.0 * M_PI * m * k / K;
            sc += c[k] * cos(arg);
            ss += c[k] * sin(arg);
        }
        mod[m] = sc * sc + ss * ss;
    }
    for (int m = 0; m < K; m++)
        if (mod[m] < 1.0e-7) mod[m] = 0.5 * (mod[(m - 1 + K) % K] + mod[(m + 1) % K]);
}

/* Grid potential phi = IFFT(G * FFT(Q)) and the reciprocal energy. */
static double pme_solve(const onb_t* s, double* grid /* complex, in: Q, out: phi */) {
    int Kx = s->grid[0], Ky = s->grid[1], Kz = s->grid[2];
    double* mx = (double*)malloc(sizeof(double) * (size_t)Kx);
    double* my = (double*)malloc(sizeof(double) * (size_t)Ky);
    double* mz = (double*)malloc(sizeof(double) * (size_t)Kz);
    bspline_moduli(Kx, s->order, mx);
    bspline_moduli(Ky, s->order, my);
    bspline_moduli(Kz, s->order, mz);
    o_fft3d(grid, s->grid, -1);
    double vol = s->box[0] * s->box[1] * s->box[2];
    double pref = ONB_ONE_4PI_EPS0 / (M_PI * vol);
    double fac = M_PI * M_PI / (s->alpha * s->alpha);
    double rb[3][3];
    recip_box(s, rb);
    double energy = 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_threads) reduction(+ : energy)
#endif
    for (int ix = 0; ix < Kx; ix++) {
        int mxi = ix <= Kx / 2 ? ix : ix - Kx;
        for (int iy = 0; iy < Ky; iy++) {
            int myi = iy <= Ky / 2 ? iy : iy - Ky;
            for (int iz = 0; iz < Kz; iz++) {
                int mzi = iz <= Kz / 2 ? iz : iz - Kz;
                /* m = mx a* + my b* + mz c*, the reciprocal vectors being the columns of rb */
                double kx = mxi * rb[0][0];
                double ky = mxi * rb[1][0] + myi * rb[1][1];
                double kz = mxi * rb[2][0] + myi * rb[2][1] + mzi * rb[2][2];
                long idx = ((long)ix * Ky + iy) * Kz + iz;
                double m2 = kx * kx + ky * ky + kz * kz;
                double G = 0.0;
                if (ix != 0 || iy != 0 || iz != 0) G = pref * exp(-fac * m2) / (m2 * mx[ix] * my[iy] * mz[iz]);
                double re = grid[2 * idx], im = grid[2 * idx + 1];
                energy += 0.5 * G * (re * re + im * im);
                grid[2 * idx] = G * re;
                grid[2 * idx + 1] = G * im;
            }
        }
    }
    o_fft3d(grid, s->grid, +1);
    free(mx);
    free(my);
    free(mz);
    return energy;
}

typedef struct {
    int base[3];
    double w[3][16], dw[3][16];
} stencil_t;

static void atom_stencil(const onb_t* s, const double* p, stencil_t* st) {
    double rb[3][3];
    recip_box(s, rb);
    for (int a = 0; a < 3; a++) {
        double f = p[0] * rb[0][a] + p[1] * rb[1][a] + p[2] * rb[2][a];
        f -= floor(f);
        double u = f * s->grid[a];
        int b = (int)floor(u);
        double t = u - b;
        if (b >= s->grid[a]) b -= s->grid[a]; /* f rounding to 1.0 */
        st->base[a] = b;
        bspline(t, s->order, st->w[a], st->dw[a]);
    }
}

/* Reciprocal energy; forces (nullable) accumulated; dUdq (nullable) receives
 * the grid potential at each particle. */
static double pme_recip(const onb_t* s, const double* pos, double* forces, double* dUdq) {
    int Kx = s->grid[0], Ky = s->grid[1], Kz = s->grid[2], n = s->order;
    long G = (long)Kx * Ky * Kz;
    double* grid = (double*)calloc((size_t)(2 * G), sizeof(double));
    for (int i = 0; i < s->n; i++) {
        double q = s->charge[i];
        if (q == 0.0) continue;
        stencil_t st;
        atom_stencil(s, pos + 3 * i, &st);
        for (int a = 0; a < n; a++) {
            int ix = (st.base[0] - a + Kx) % Kx;
            for (int b = 0; b < n; b++) {
                int iy = (st.base[1] - b + Ky) % Ky;
                double wab = q * st.w[0][a] * st.w[1][b];
                for (int c = 0; c < n; c++) {
                    int iz = (st.base[2] - c + Kz) % Kz;
                    grid[2 * (((long)ix * Ky + iy) * Kz + iz)] += wab * st.w[2][c];
                }
            }
        }
    }
    double energy = pme_solve(s, grid);
    if (forces || dUdq) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_threads)
#endif
        for (int i = 0; i < s->n; i++) {
            double q = s->charge[i];
            stencil_t st;
            atom_stencil(s, pos + 3 * i, &st);
            double gx = 0.0, gy = 0.0, gz = 0.0, phi = 0.0;
            for (int a = 0; a < n; a++) {
                int ix = (st.base[0] - a + Kx) % Kx;
                for (int b = 0; b < n; b++) {
                    int iy = (st.base[1] - b + Ky) % Ky;
                    for (int c = 0; c < n; c++) {
                        int iz = (st.base[2] - c + Kz) % Kz;
                        double v = grid[2 * (((long)ix * Ky + iy) * Kz + iz)];
                        gx += st.dw[0][a] * st.w[1][b] * st.w[2][c] * v;
                        gy += st.w[0][a] * st.dw[1][b] * st.w[2][c] * v;
                        gz += st.w[0][a] * st.w[1][b] * st.dw[2][c] * v;
                        phi += st.w[0][a] * st.w[1][b] * st.w[2][c] * v;
                    }
                }
            }
            if (forces) {
                /* -q grad phi: d(grid coordinate d)/dx_j = K_d rb[j][d] */
                double rb[3][3];
                recip_box(s, rb);
                const double g[3] = {gx * Kx, gy * Ky, gz * Kz};
                for (int j = 0; j < 3; j++)
                    forces[3 * i + j] -= q * (g[0] * rb[j][0] + g[1] * rb[j][1] + g[2] * rb[j][2]);
            }
            if (dUdq) dUdq[i] += phi;
        }
    }
    free(grid);
    return energy;
}

int onb_ewald_recip_exact(const onb_t* s, const double* pos, int kmax, double* energy, double* forces) {
    double vol = s->box[0] * s->box[1] * s->box[2];
    double rb[3][3];
    recip_box(s, rb);
    double fac = M_PI * M_PI / (s->alpha * s->alpha);
    double e = 0.0;
    if (forces) memset(forces, 0, sizeof(double) * 3 * (size_t)s->n);
    double* cs = (double*)malloc(sizeof(double) * (size_t)s->n);
    double* sn = (double*)malloc(sizeof(double) * (size_t)s->n);
    for (int mx = -kmax; mx <= kmax; mx++)
        for (int my = -kmax; my <= kmax; my++)
            for (int mz = -kmax; mz <= kmax; mz++) {
                if (mx == 0 && my == 0 && mz == 0) continue;
                double k[3] = {mx * rb[0][0], mx * rb[1][0] + my * rb[1][1],
                               mx * rb[2][0] + my * rb[2][1] + mz * rb[2][2]};
                double m2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
                double f = exp(-fac * m2) / m2;
                double sr = 0.0, si = 0.0;
                for (int j = 0; j < s->n; j++) {
                    double th = 2.0 * M_PI * (k[0] * pos[3 * j] + k[1] * pos[3 * j + 1] + k[2] * pos[3 * j + 2]);
                    cs[j] = cos(th);
                    sn[j] = sin(th);
                    sr += s->charge[j] * cs[j];
                    si += s->charge[j] * sn[j];
                }
                e += f * (sr * sr + si * si);
                if (forces) {
                    /* F_j = (2 k_e / V) f q_j k Im(e^{i th_j} conj(S)) */
                    for (int j = 0; j < s->n; j++) {
                        double im = sn[j] * sr - cs[j] * si;
                        double c = 2.0 * ONB_ONE_4PI_EPS0 / vol * f * s->charge[j] * im;
                        forces[3 * j] += c * k[0];
                        forces[3 * j + 1] += c * k[1];
                        forces[3 * j + 2] += c * k[2];
                    }
                }
            }
    free(cs);
    free(sn);
    *energy = ONB_ONE_4PI_EPS0 / (2.0 * M_PI * vol) * e;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Public evaluators                                                           */
/* ------------------------------------------------------------------------- */

int onb_energy_forces(const onb_t* s, const double* pos, const double* pos_cut, double* energy, double* forces,
                      oterms_t* terms) {
    if (s->n <= 0) return -1;
    excl_csr ex;
    if (build_excl(s, &ex)) return -2;
    if (forces) memset(forces, 0, sizeof(double) * 3 * (size_t)s->n);
    direct_job J = {s, pos, pos_cut ? pos_cut : pos, &ex, forces, NULL, NULL, NULL, is_triclinic(s)};
    oterms_t t = {0, 0, 0, 0, 0};
    t.direct = direct_space(&J);
    t.exceptions = exceptions_term(s, pos, forces, NULL, NULL, NULL);
    if (s->method == ONB_PME) {
        t.recip = pme_recip(s, pos, forces, NULL);
        double q2 = 0.0;
        for (int i = 0; i < s->n; i++) q2 += s->charge[i] * s->charge[i];
        t.self = -ONB_ONE_4PI_EPS0 * s->alpha / sqrt(M_PI) * q2;
    }
    t.disp = dispersion_correction(s);
    free_excl(&ex);
    if (terms) *terms = t;
    if (energy) *energy = t.direct + t.exceptions + t.recip + t.self + t.disp;
    return 0;
}

int onb_param_derivs(const onb_t* s, const double* pos, const double* pos_cut, double* dUdq, double* dUdsig,
                     double* dUdeps) {
    excl_csr ex;
    if (build_excl(s, &ex)) return -2;
    if (dUdq) memset(dUdq, 0, sizeof(double) * (size_t)s->n);
    if (dUdsig) memset(dUdsig, 0, sizeof(double) * (size_t)s->n);
    if (dUdeps) memset(dUdeps, 0, sizeof(double) * (size_t)s->n);
    direct_job J = {s, pos, pos_cut ? pos_cut : pos, &ex, NULL, dUdq, dUdsig, dUdeps, is_triclinic(s)};
    direct_space(&J);
    /* exceptions with explicit chargeProd do not depend on the particle charges
       except through the PME exclusion correction */
    exceptions_term(s, pos, NULL, dUdq, NULL, NULL);
    if (s->method == ONB_PME && dUdq) {
        pme_recip(s, pos, NULL, dUdq);
        for (int i = 0; i < s->n; i++) dUdq[i] += -2.0 * ONB_ONE_4PI_EPS0 * s->alpha / sqrt(M_PI) * s->charge[i];
    }
    free_excl(&ex);
    return 0;
}

double o_softcore(double u, double umax, double a, double ub, double* fp) {
    /* ReferenceATMMetaForceKernels.cpp:26-37 */
    if (u <= ub) {
        *fp = 1.0;
        return u;
    }
    double gu = (u - ub) / (a * (umax - ub));
    double zeta = 1.0 + 2.0 * gu * (gu + 1.0);
    double zetap = pow(zeta, a);
    double sfac = 4.0 * (2.0 * gu + 1.0) / zeta;
    *fp = sfac * zetap / pow(1.0 + zetap, 2);
    return (umax - ub) * (zetap - 1.0) / (zetap + 1.0) + ub;
}

void o_atm_merge(double E1, double E2, const double* p, int n, const double* F1, const double* F2, double* f_out,
                 double* out) {
    /* ReferenceATMMetaForceKernels.cpp:56-113 */
    double lambda1 = p[0], lambda2 = p[1], alpha = p[2], u0 = p[3], w0 = p[4];
    double umax = p[5], ubcore = p[6], acore = p[7], direction = p[8];
    double fp;
    double u = direction > 0 ? E2 - E1 : E1 - E2;
    double e0 = direction > 0 ? E1 : E2;
    double usc = o_softcore(u, umax, acore, ubcore, &fp);
    double ebias = 0.0;
    double ee = 1.0 + exp(-alpha * (usc - u0));
    if (alpha > 0) ebias = ((lambda2 - lambda1) / alpha) * log(ee);
    ebias += lambda2 * usc + w0;
    double bfp = (lambda2 - lambda1) / ee + lambda1;
    double energy = e0 + ebias;
    double sp = bfp * fp;
    if (f_out) {
        for (int k = 0; k < 3 * n; k++)
            f_out[k] = direction > 0 ? sp * F2[k] + (1.0 - sp) * F1[k] : sp * F1[k] + (1.0 - sp) * F2[k];
    }
    out[0] = energy;
    out[1] = usc;
    out[2] = sp;
    out[3] = ebias;
    out[4] = u;
    out[5] = e0;
    out[6] = bfp;
    out[7] = fp;
}

void o_softplus_param_grad(double usc, const double* p, double* dW) {
    double l1 = p[0], l2 = p[1], alpha = p[2], u0 = p[3];
    double x = exp(-alpha * (usc - u0));
    double ee = 1.0 + x;
    if (alpha > 0) {
        double L = log(ee);
        dW[0] = -L / alpha;
        dW[1] = L / alpha + usc;
        dW[2] = -(l2 - l1) / (alpha * alpha) * L - (l2 - l1) / alpha * (usc - u0) * x / ee;
        dW[3] = (l2 - l1) * x / ee;
    } else {
        dW[0] = 0.0;
        dW[1] = usc;
        dW[2] = 0.0;
        dW[3] = 0.0;
    }
    dW[4] = 1.0;
}

int o_atm_eval(const onb_t* s, const double* pos, const double* displ, const double* params, const double* pos_cut,
               double* forces, double* out, double* E12, double* F12) {
    int n = s->n;
    double* pos2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* pc2 = pos_cut ? (double*)malloc(sizeof(double) * 3 * (size_t)n) : NULL;
    double* F1 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    double* F2 = (double*)malloc(sizeof(double) * 3 * (size_t)n);
    /* ReferenceATMMetaForceKernels.cpp:116-124: pos2 = pos + displacement */
    for (int k = 0; k < 3 * n; k++) {
        pos2[k] = pos[k] + displ[k];
        if (pc2) pc2[k] = pos_cut[k] + displ[k];
    }
    double E1, E2;
    int rc = onb_energy_forces(s, pos, pos_cut, &E1, F1, NULL);
    if (!rc) rc = onb_energy_forces(s, pos2, pc2, &E2, F2, NULL);
    if (!rc) {
        o_atm_merge(E1, E2, params, n, F1, F2, forces, out);
        if (E12) {
            E12[0] = E1;
            E12[1] = E2;
        }
        if (F12) {
            memcpy(F12, F1, sizeof(double) * 3 * (size_t)n);
            memcpy(F12 + 3 * (size_t)n, F2, sizeof(double) * 3 * (size_t)n);
        }
    }
    free(pos2);
    free(pc2);
    free(F1);
    free(F2);
    return rc;
}

static int legal_size(int n) {
    for (;; n++) {
        int m = n;
        int primes[4] = {2, 3, 5, 7};
        for (int k = 0; k < 4; k++)
            while (m % primes[k] == 0) m /= primes[k];
        if (m == 1) return n;
    }
}

void o_pme_parameters(double cutoff, double tol, const double* box, int legal, double* alpha, int* grid) {
    *alpha = sqrt(-log(2.0 * tol)) / cutoff;
    for (int a = 0; a < 3; a++) {
        int g = (int)ceil(2.0 * (*alpha) * box[a] / (3.0 * pow(tol, 0.2)));
        if (g < 6) g = 6;
        grid[a] = legal ? legal_size(g) : g;
    }
}
