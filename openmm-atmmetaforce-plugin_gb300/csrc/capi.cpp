// extern "C" entry points of include/atm_capi.h.
//
// Every entry point converts C++ exceptions into ATM_* status codes and a
// thread-local message, the way the reference's SWIG layer turns C++
// exceptions into Python exceptions (python/atmmetaforceplugin.i:54-61).
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/atm_capi.h"
#include "engine.h"
#include "md.h"
#include "model.h"

using namespace atm;

struct atm_force_s {
    std::unique_ptr<ATMMetaForce> f;
    bool owned_by_system = false;
};
struct atm_nonbonded_s {
    std::unique_ptr<NonbondedForce> nb;
    bool owned_by_system = false;
};
struct atm_system_s {
    System sys;
    atm_force_t atm_handle = nullptr;
    atm_nonbonded_t nb_handle = nullptr;
};

struct atm_context_s {
    std::unique_ptr<Engine> eng;
    int atm_group = 0, nb_group = 0;
    bool var_nb = true;
    int n = 0;
    std::vector<int> particle_ids;  // ATMMetaForce particle field at creation
    bool positions_set = false;
    bool dirty = true;
    double pert = 0.0;
    std::vector<double> forces, forces_nb;
    std::vector<double> results;
};

struct atm_batch_s {
    std::unique_ptr<Engine> eng;
    std::vector<double> results;
    std::vector<double> matrix;
    bool evaluated = false;
    double* scratch = nullptr;  // device staging of the host backward()
    size_t scratch_n = 0;
    ~atm_batch_s() {
        if (scratch) cudaFree(scratch);
    }
};

struct atm_md_s {
    std::unique_ptr<MDDriver> md;
};

static thread_local std::string g_error;

namespace atm {
void set_last_error(const std::string& msg) { g_error = msg; }
}  // namespace atm

#define API_BEGIN try {
#define API_END                                    \
    g_error.clear();                               \
    return ATM_OK;                                 \
    }                                              \
    catch (const Error& e) {                       \
        g_error = e.what();                        \
        return e.code;                             \
    }                                              \
    catch (const std::exception& e) {              \
        g_error = e.what();                        \
        return ATM_ERR_INVALID_ARGUMENT;           \
    }                                              \
    catch (...) {                                  \
        g_error = "unknown error";                 \
        return ATM_ERR_INVALID_ARGUMENT;           \
    }

#define REQUIRE(cond, code, msg) \
    if (!(cond)) throw Error(code, msg)

static std::map<std::string, std::string> parse_props(const char* p) {
    std::map<std::string, std::string> m;
    if (!p) return m;
    std::stringstream ss(p);
    std::string item;
    while (std::getline(ss, item, ';')) {
        auto eq = item.find('=');
        if (eq == std::string::npos) continue;
        m[item.substr(0, eq)] = item.substr(eq + 1);
    }
    return m;
}

static bool prop_bool(const std::map<std::string, std::string>& m, const char* key, bool def) {
    auto it = m.find(key);
    if (it == m.end()) return def;
    const std::string& v = it->second;
    if (v == "1" || v == "true" || v == "True") return true;
    if (v == "0" || v == "false" || v == "False") return false;
    throw Error(ATM_ERR_INVALID_ARGUMENT, std::string("Bad value for property ") + key + ": " + v);
}

static double prop_double(const std::map<std::string, std::string>& m, const char* key, double def);

// SpreadBrick=n: the PME spreading brick edge in grid points (0: per atom), as the
// autotuner would choose it; absent: the engine's default until a tuning.
static void apply_spread_brick(Engine& e, const std::map<std::string, std::string>& m) {
    if (m.count("SpreadBrick")) e.set_spread_brick((int)prop_double(m, "SpreadBrick", 16.0));
}

static double prop_double(const std::map<std::string, std::string>& m, const char* key, double def) {
    auto it = m.find(key);
    if (it == m.end()) return def;
    try {
        size_t used = 0;
        double v = std::stod(it->second, &used);
        if (used == it->second.size()) return v;
    } catch (...) {
    }
    throw Error(ATM_ERR_INVALID_ARGUMENT, std::string("Bad value for property ") + key + ": " + it->second);
}

extern "C" {

const char* atm_last_error(void) { return g_error.c_str(); }
const char* atm_version(void) { return kVersion; }
const char* atm_global_name(int which) { return global_name(which); }

// ---- ATMMetaForce ---------------------------------------------------------

int atm_force_create(double lambda1, double lambda2, double alpha, double u0, double w0, double umax, double ubcore,
                     double acore, double direction, const int* groups, int n_groups, atm_force_t* out) {
    API_BEGIN
    REQUIRE(out, ATM_ERR_INVALID_ARGUMENT, "null output handle");
    REQUIRE(n_groups >= 0 && (n_groups == 0 || groups), ATM_ERR_INVALID_ARGUMENT, "bad variable group list");
    std::vector<int> g(groups, groups + n_groups);
    auto* h = new atm_force_s;
    h->f.reset(new ATMMetaForce(lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction, g));
    *out = h;
    API_END
}

int atm_force_destroy(atm_force_t force) {
    API_BEGIN
    if (!force) return ATM_OK;
    REQUIRE(!force->owned_by_system, ATM_ERR_STATE, "the force is owned by a System");
    delete force;
    API_END
}

int atm_force_add_particle(atm_force_t force, int particle, double dx, double dy, double dz, int* index) {
    API_BEGIN
    REQUIRE(force, ATM_ERR_INVALID_ARGUMENT, "null force");
    int k = force->f->addParticle(particle, dx, dy, dz);
    if (index) *index = k;
    API_END
}

int atm_force_get_particle_parameters(atm_force_t force, int index, int* particle, double* dx, double* dy, double* dz) {
    API_BEGIN
    REQUIRE(force && particle && dx && dy && dz, ATM_ERR_INVALID_ARGUMENT, "null argument");
    force->f->getParticleParameters(index, *particle, *dx, *dy, *dz);
    API_END
}

int atm_force_set_particle_parameters(atm_force_t force, int index, int particle, double dx, double dy, double dz) {
    API_BEGIN
    REQUIRE(force, ATM_ERR_INVALID_ARGUMENT, "null force");
    force->f->setParticleParameters(index, particle, dx, dy, dz);
    API_END
}

int atm_force_get_num_particles(atm_force_t force, int* n) {
    API_BEGIN
    REQUIRE(force && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = force->f->getNumParticles();
    API_END
}

int atm_force_get_default(atm_force_t force, int which, double* value) {
    API_BEGIN
    REQUIRE(force && value, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(which >= 0 && which < NUM_GLOBALS, ATM_ERR_INDEX, "unknown parameter index");
    *value = force->f->getDefault(which);
    API_END
}

int atm_force_get_variable_force_groups(atm_force_t force, int* groups, int cap, int* n) {
    API_BEGIN
    REQUIRE(force && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    const auto& g = force->f->getVariableForceGroups();
    *n = (int)g.size();
    for (int k = 0; k < (int)g.size() && k < cap; k++) groups[k] = g[k];
    API_END
}

int atm_force_set_force_group(atm_force_t force, int group) {
    API_BEGIN
    REQUIRE(force, ATM_ERR_INVALID_ARGUMENT, "null force");
    force->f->setForceGroup(group);
    API_END
}

int atm_force_get_force_group(atm_force_t force, int* group) {
    API_BEGIN
    REQUIRE(force && group, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *group = force->f->getForceGroup();
    API_END
}

int atm_force_set_name(atm_force_t force, const char* name) {
    API_BEGIN
    REQUIRE(force && name, ATM_ERR_INVALID_ARGUMENT, "null argument");
    force->f->setName(name);
    API_END
}

static void copy_string(const std::string& s, char* buf, size_t cap, size_t* len) {
    if (len) *len = s.size();
    if (buf && cap > 0) {
        size_t k = s.size() < cap - 1 ? s.size() : cap - 1;
        std::memcpy(buf, s.data(), k);
        buf[k] = '\0';
    }
}

int atm_force_get_name(atm_force_t force, char* buf, size_t cap, size_t* len) {
    API_BEGIN
    REQUIRE(force, ATM_ERR_INVALID_ARGUMENT, "null force");
    copy_string(force->f->getName(), buf, cap, len);
    API_END
}

int atm_force_uses_periodic_boundary_conditions(atm_force_t force, int* uses) {
    API_BEGIN
    REQUIRE(force && uses, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *uses = 0;  // ATMMetaForce.h:135-137
    API_END
}

int atm_force_update_parameters_in_context(atm_force_t force, atm_context_t ctx) {
    API_BEGIN
    REQUIRE(force && ctx, ATM_ERR_INVALID_ARGUMENT, "null argument");
    const ATMMetaForce& f = *force->f;
    // ReferenceATMMetaForceKernels.cpp:146-154: the particle count and indices may not change
    REQUIRE(f.getNumParticles() == ctx->n, ATM_ERR_PARTICLES,
            "copyParametersToContext: The number of ATMMetaForce particles has changed");
    std::vector<double> d(3 * (size_t)ctx->n);
    for (int i = 0; i < ctx->n; i++) {
        REQUIRE(f.particles[i].particle == ctx->particle_ids[i], ATM_ERR_PARTICLES,
                "copyParametersToContext: A particle index has changed");
        d[3 * i] = f.particles[i].dx;
        d[3 * i + 1] = f.particles[i].dy;
        d[3 * i + 2] = f.particles[i].dz;
    }
    ctx->eng->set_displacements(0, d.data());
    ctx->dirty = true;
    API_END
}

int atm_force_get_perturbation_energy(atm_force_t force, atm_context_t ctx, double* value) {
    API_BEGIN
    REQUIRE(force && ctx && value, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *value = ctx->pert;
    API_END
}

int atm_force_serialize(atm_force_t force, char* buf, size_t cap, size_t* len) {
    API_BEGIN
    REQUIRE(force, ATM_ERR_INVALID_ARGUMENT, "null force");
    copy_string(serialize(*force->f), buf, cap, len);
    API_END
}

int atm_force_deserialize(const char* xml, atm_force_t* out) {
    API_BEGIN
    REQUIRE(xml && out, ATM_ERR_INVALID_ARGUMENT, "null argument");
    auto f = deserialize(xml);
    auto* h = new atm_force_s;
    h->f = std::move(f);
    *out = h;
    API_END
}

// ---- NonbondedForce -------------------------------------------------------

int atm_nonbonded_create(atm_nonbonded_t* out) {
    API_BEGIN
    REQUIRE(out, ATM_ERR_INVALID_ARGUMENT, "null output handle");
    auto* h = new atm_nonbonded_s;
    h->nb.reset(new NonbondedForce);
    *out = h;
    API_END
}

int atm_nonbonded_destroy(atm_nonbonded_t nb) {
    API_BEGIN
    if (!nb) return ATM_OK;
    REQUIRE(!nb->owned_by_system, ATM_ERR_STATE, "the force is owned by a System");
    delete nb;
    API_END
}

int atm_nonbonded_add_particle(atm_nonbonded_t nb, double charge, double sigma, double epsilon, int* index) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    int k = nb->nb->addParticle(charge, sigma, epsilon);
    if (index) *index = k;
    API_END
}

int atm_nonbonded_set_particle_parameters(atm_nonbonded_t nb, int index, double charge, double sigma, double epsilon) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(index >= 0 && index < (int)nb->nb->charge.size(), ATM_ERR_INDEX, "Index out of range");
    nb->nb->charge[index] = charge;
    nb->nb->sigma[index] = sigma;
    nb->nb->epsilon[index] = epsilon;
    API_END
}

int atm_nonbonded_get_particle_parameters(atm_nonbonded_t nb, int index, double* charge, double* sigma,
                                          double* epsilon) {
    API_BEGIN
    REQUIRE(nb && charge && sigma && epsilon, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(index >= 0 && index < (int)nb->nb->charge.size(), ATM_ERR_INDEX, "Index out of range");
    *charge = nb->nb->charge[index];
    *sigma = nb->nb->sigma[index];
    *epsilon = nb->nb->epsilon[index];
    API_END
}

int atm_nonbonded_get_num_particles(atm_nonbonded_t nb, int* n) {
    API_BEGIN
    REQUIRE(nb && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = (int)nb->nb->charge.size();
    API_END
}

int atm_nonbonded_add_exception(atm_nonbonded_t nb, int i, int j, double charge_prod, double sigma, double epsilon,
                                int* index) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(i >= 0 && j >= 0, ATM_ERR_INDEX, "Index out of range");
    int k = nb->nb->addException(i, j, charge_prod, sigma, epsilon);
    if (index) *index = k;
    API_END
}

int atm_nonbonded_get_num_exceptions(atm_nonbonded_t nb, int* n) {
    API_BEGIN
    REQUIRE(nb && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = (int)nb->nb->exceptions.size();
    API_END
}

int atm_nonbonded_set_method(atm_nonbonded_t nb, int method) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(method == 0 || method == 1 || method == 2 || method == 4, ATM_ERR_UNSUPPORTED,
            "Unsupported nonbonded method");
    nb->nb->method = method;
    API_END
}

int atm_nonbonded_set_cutoff(atm_nonbonded_t nb, double cutoff) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(cutoff > 0, ATM_ERR_INVALID_ARGUMENT, "The cutoff must be positive");
    nb->nb->cutoff = cutoff;
    API_END
}

int atm_nonbonded_set_reaction_field_dielectric(atm_nonbonded_t nb, double eps_rf) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    nb->nb->epsRF = eps_rf;
    API_END
}

int atm_nonbonded_set_ewald_error_tolerance(atm_nonbonded_t nb, double tol) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(tol > 0 && tol < 0.5, ATM_ERR_INVALID_ARGUMENT, "Bad Ewald error tolerance");
    nb->nb->ewaldTol = tol;
    API_END
}

int atm_nonbonded_set_pme_parameters(atm_nonbonded_t nb, double alpha, int nx, int ny, int nz) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    nb->nb->alpha = alpha;
    nb->nb->grid[0] = nx;
    nb->nb->grid[1] = ny;
    nb->nb->grid[2] = nz;
    API_END
}

int atm_nonbonded_set_use_dispersion_correction(atm_nonbonded_t nb, int use) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    nb->nb->dispersionCorrection = use != 0;
    API_END
}

int atm_nonbonded_set_force_group(atm_nonbonded_t nb, int group) {
    API_BEGIN
    REQUIRE(nb, ATM_ERR_INVALID_ARGUMENT, "null force");
    REQUIRE(group >= 0 && group <= 31, ATM_ERR_INVALID_ARGUMENT, "Force group must be between 0 and 31");
    nb->nb->forceGroup = group;
    API_END
}

int atm_nonbonded_get_force_group(atm_nonbonded_t nb, int* group) {
    API_BEGIN
    REQUIRE(nb && group, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *group = nb->nb->forceGroup;
    API_END
}

// ---- System ---------------------------------------------------------------

int atm_system_create(atm_system_t* out) {
    API_BEGIN
    REQUIRE(out, ATM_ERR_INVALID_ARGUMENT, "null output handle");
    *out = new atm_system_s;
    API_END
}

int atm_system_destroy(atm_system_t sys) {
    API_BEGIN
    if (!sys) return ATM_OK;
    if (sys->atm_handle) {
        sys->atm_handle->f.release();  // the System's unique_ptr owns the object
        delete sys->atm_handle;
    }
    if (sys->nb_handle) {
        sys->nb_handle->nb.release();
        delete sys->nb_handle;
    }
    delete sys;
    API_END
}

int atm_system_add_particle(atm_system_t sys, double mass, int* index) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    int k = sys->sys.addParticle(mass);
    if (index) *index = k;
    API_END
}

int atm_system_get_num_particles(atm_system_t sys, int* n) {
    API_BEGIN
    REQUIRE(sys && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = (int)sys->sys.masses.size();
    API_END
}

// Box vectors in OpenMM's reduced form (System::setDefaultPeriodicBoxVectors):
// a = (ax, 0, 0), b = (bx, by, 0), c = (cx, cy, cz) with ax, by, cz > 0,
// |bx| <= ax/2, |cx| <= ax/2, |cy| <= by/2.  box = (ax, by, cz), tilt = (bx, cx, cy).
static void read_box(const double* a, const double* b, const double* c, double* box, double* tilt) {
    REQUIRE(a && b && c, ATM_ERR_INVALID_ARGUMENT, "null box vector");
    REQUIRE(a[1] == 0 && a[2] == 0 && b[2] == 0, ATM_ERR_INVALID_ARGUMENT,
            "First periodic box vector must be parallel to x, the second must lie in the xy plane");
    REQUIRE(a[0] > 0 && b[1] > 0 && c[2] > 0, ATM_ERR_INVALID_ARGUMENT, "Box vectors must be positive");
    REQUIRE(std::fabs(b[0]) <= 0.5 * a[0] * (1 + 1e-12) && std::fabs(c[0]) <= 0.5 * a[0] * (1 + 1e-12) &&
                std::fabs(c[1]) <= 0.5 * b[1] * (1 + 1e-12),
            ATM_ERR_INVALID_ARGUMENT, "Triclinic box vectors must be in reduced form");
    box[0] = a[0];
    box[1] = b[1];
    box[2] = c[2];
    tilt[0] = b[0];
    tilt[1] = c[0];
    tilt[2] = c[1];
}

int atm_system_set_default_periodic_box_vectors(atm_system_t sys, const double* a, const double* b, const double* c) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    read_box(a, b, c, sys->sys.box, sys->sys.tilt);
    API_END
}

int atm_system_add_nonbonded(atm_system_t sys, atm_nonbonded_t nb) {
    API_BEGIN
    REQUIRE(sys && nb, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(!nb->owned_by_system, ATM_ERR_STATE, "The force already belongs to a System");
    REQUIRE(!sys->sys.nonbonded, ATM_ERR_UNSUPPORTED, "Only one NonbondedForce per System is supported");
    sys->sys.nonbonded.reset(nb->nb.get());
    nb->owned_by_system = true;
    sys->nb_handle = nb;
    API_END
}

int atm_system_add_atm_force(atm_system_t sys, atm_force_t force) {
    API_BEGIN
    REQUIRE(sys && force, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(!force->owned_by_system, ATM_ERR_STATE, "The force already belongs to a System");
    REQUIRE(!sys->sys.atm, ATM_ERR_UNSUPPORTED, "Only one ATMMetaForce per System is supported");
    sys->sys.atm.reset(force->f.get());
    force->owned_by_system = true;
    sys->atm_handle = force;
    API_END
}

// ---- MD terms of a System --------------------------------------------------

static void check_particle(const System& s, int i) {
    REQUIRE(i >= 0 && i < (int)s.masses.size(), ATM_ERR_INDEX, "Particle index out of range");
}

int atm_system_add_constraint(atm_system_t sys, int i, int j, double distance, int* index) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    check_particle(sys->sys, i);
    check_particle(sys->sys, j);
    REQUIRE(i != j && distance > 0.0, ATM_ERR_INVALID_ARGUMENT, "Invalid constraint");
    sys->sys.constraints.push_back({i, j, distance});
    if (index) *index = (int)sys->sys.constraints.size() - 1;
    API_END
}

int atm_system_get_num_constraints(atm_system_t sys, int* n) {
    API_BEGIN
    REQUIRE(sys && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = (int)sys->sys.constraints.size();
    API_END
}

int atm_system_add_bond(atm_system_t sys, int i, int j, double length, double k) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    check_particle(sys->sys, i);
    check_particle(sys->sys, j);
    sys->sys.bonds.push_back({i, j, length, k});
    API_END
}

int atm_system_add_angle(atm_system_t sys, int i, int j, int l, double angle, double k) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    check_particle(sys->sys, i);
    check_particle(sys->sys, j);
    check_particle(sys->sys, l);
    sys->sys.angles.push_back({i, j, l, angle, k});
    API_END
}

int atm_system_add_centroid_restraint(atm_system_t sys, int n1, const int* g1, int n2, const int* g2, double kf,
                                      double tol, const double* offset) {
    API_BEGIN
    REQUIRE(sys && g1 && g2 && n1 > 0 && n2 > 0, ATM_ERR_INVALID_ARGUMENT, "empty centroid group");
    CentroidRestraint c;
    for (int k = 0; k < n1; k++) {
        check_particle(sys->sys, g1[k]);
        c.g1.push_back(g1[k]);
    }
    for (int k = 0; k < n2; k++) {
        check_particle(sys->sys, g2[k]);
        c.g2.push_back(g2[k]);
    }
    c.kf = kf;
    c.tol = tol;
    for (int k = 0; k < 3; k++) c.offset[k] = offset ? offset[k] : 0.0;
    sys->sys.centroid_restraints.push_back(c);
    API_END
}

int atm_system_add_position_restraint(atm_system_t sys, int particle, double x0, double y0, double z0, double fc,
                                      double tol) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    check_particle(sys->sys, particle);
    sys->sys.position_restraints.push_back({particle, x0, y0, z0, fc, tol});
    API_END
}

int atm_system_set_position_restraints_periodic(atm_system_t sys, int periodic) {
    API_BEGIN
    REQUIRE(sys, ATM_ERR_INVALID_ARGUMENT, "null system");
    sys->sys.position_restraints_periodic = periodic != 0;
    API_END
}

// ---- Context --------------------------------------------------------------

int atm_context_create(atm_system_t sys, int device, const char* properties, atm_context_t* out) {
    API_BEGIN
    REQUIRE(sys && out, ATM_ERR_INVALID_ARGUMENT, "null argument");
    auto props = parse_props(properties);
    bool diff = prop_bool(props, "DifferencePath", false);
    ReplicaSpec spec = spec_from_system(sys->sys);
    std::unique_ptr<atm_context_s> c(new atm_context_s);
    c->atm_group = sys->sys.atm->getForceGroup();
    c->nb_group = sys->sys.nonbonded->forceGroup;
    c->var_nb = spec.var_nb;
    c->n = spec.n;
    for (const auto& p : sys->sys.atm->particles) c->particle_ids.push_back(p.particle);
    std::vector<ReplicaSpec> v;
    v.push_back(std::move(spec));
    c->eng.reset(new Engine(std::move(v), device, !diff));
    c->eng->set_list_skin(prop_double(props, "ListSkin", 0.0));
    c->eng->set_fused(prop_bool(props, "FusedTiles", false));
    c->eng->set_spread_owner(prop_bool(props, "SpreadByOwner", true));
    apply_spread_brick(*c->eng, props);
    c->forces.resize(3 * (size_t)c->n);
    c->forces_nb.resize(3 * (size_t)c->n);
    c->results.resize(NUM_RES);
    *out = c.release();
    API_END
}

int atm_context_destroy(atm_context_t ctx) {
    API_BEGIN
    delete ctx;
    API_END
}

int atm_context_set_positions(atm_context_t ctx, const double* pos, int n) {
    API_BEGIN
    REQUIRE(ctx && pos, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(n == ctx->n, ATM_ERR_INVALID_ARGUMENT, "Called setPositions() on a Context with the wrong number of positions");
    ctx->eng->set_positions(0, pos);
    ctx->positions_set = true;
    ctx->dirty = true;
    API_END
}

int atm_context_set_periodic_box_vectors(atm_context_t ctx, const double* a, const double* b, const double* c) {
    API_BEGIN
    REQUIRE(ctx, ATM_ERR_INVALID_ARGUMENT, "null context");
    double box[3], tilt[3];
    read_box(a, b, c, box, tilt);
    ctx->eng->set_box(0, box, tilt);
    ctx->dirty = true;
    API_END
}

int atm_context_set_parameter(atm_context_t ctx, const char* name, double value) {
    API_BEGIN
    REQUIRE(ctx && name, ATM_ERR_INVALID_ARGUMENT, "null argument");
    int k = global_index(name);
    REQUIRE(k >= 0, ATM_ERR_INVALID_ARGUMENT, std::string("Called setParameter() with invalid parameter name: ") + name);
    ctx->eng->set_param(0, k, value);
    ctx->dirty = true;
    API_END
}

int atm_context_get_parameter(atm_context_t ctx, const char* name, double* value) {
    API_BEGIN
    REQUIRE(ctx && name && value, ATM_ERR_INVALID_ARGUMENT, "null argument");
    int k = global_index(name);
    REQUIRE(k >= 0, ATM_ERR_INVALID_ARGUMENT, std::string("Called getParameter() with invalid parameter name: ") + name);
    *value = ctx->eng->param(0, k);
    API_END
}

int atm_context_get_state(atm_context_t ctx, int groups_mask, double* energy, double* forces) {
    API_BEGIN
    REQUIRE(ctx, ATM_ERR_INVALID_ARGUMENT, "null context");
    REQUIRE(ctx->positions_set, ATM_ERR_STATE, "Particle positions have not been set");
    bool want_atm = (groups_mask >> ctx->atm_group) & 1;
    bool want_nb = (groups_mask >> ctx->nb_group) & 1;
    if ((want_atm || want_nb) && ctx->dirty) {
        ctx->eng->evaluate(nullptr, ctx->forces.data(), ctx->forces_nb.data(), ctx->results.data(), nullptr);
        ctx->dirty = false;
    }
    // ATMMetaForceImpl.cpp:103,125: the perturbation energy is refreshed only when the ATM group is evaluated
    if (want_atm) ctx->pert = ctx->results[RES_PERT];
    double e = 0.0;
    if (want_atm) e += ctx->results[RES_ENERGY];
    if (want_nb) e += ctx->results[RES_E1];
    if (energy) *energy = e;
    if (forces) {
        for (size_t k = 0; k < ctx->forces.size(); k++)
            forces[k] = (want_atm ? ctx->forces[k] : 0.0) + (want_nb ? ctx->forces_nb[k] : 0.0);
    }
    API_END
}

int atm_context_get_results(atm_context_t ctx, double* results) {
    API_BEGIN
    REQUIRE(ctx && results, ATM_ERR_INVALID_ARGUMENT, "null argument");
    std::memcpy(results, ctx->results.data(), sizeof(double) * NUM_RES);
    API_END
}

// ---- Batch ----------------------------------------------------------------

int atm_batch_create(const atm_system_t* systems, int n_replicas, int device, const char* properties,
                     atm_batch_t* out) {
    API_BEGIN
    REQUIRE(systems && out && n_replicas > 0, ATM_ERR_INVALID_ARGUMENT, "bad argument");
    auto props = parse_props(properties);
    bool diff = prop_bool(props, "DifferencePath", true);
    bool adjoint = prop_bool(props, "Adjoint", false);
    std::vector<ReplicaSpec> v;
    for (int r = 0; r < n_replicas; r++) {
        REQUIRE(systems[r], ATM_ERR_INVALID_ARGUMENT, "null system");
        v.push_back(spec_from_system(systems[r]->sys));
    }
    std::unique_ptr<atm_batch_s> b(new atm_batch_s);
    b->eng.reset(new Engine(std::move(v), device, !diff, adjoint));
    b->eng->set_list_skin(prop_double(props, "ListSkin", 0.0));
    b->eng->set_fused(prop_bool(props, "FusedTiles", false));
    b->eng->set_spread_owner(prop_bool(props, "SpreadByOwner", true));
    apply_spread_brick(*b->eng, props);
    b->results.resize((size_t)NUM_RES * n_replicas);
    b->matrix.resize((size_t)n_replicas * n_replicas);
    *out = b.release();
    API_END
}

int atm_batch_destroy(atm_batch_t b) {
    API_BEGIN
    delete b;
    API_END
}

int atm_batch_get_num_replicas(atm_batch_t b, int* r) {
    API_BEGIN
    REQUIRE(b && r, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *r = b->eng->replicas();
    API_END
}

int atm_batch_get_num_particles(atm_batch_t b, int replica, int* n) {
    API_BEGIN
    REQUIRE(b && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(replica >= 0 && replica < b->eng->replicas(), ATM_ERR_INDEX, "Replica index out of range");
    *n = b->eng->atoms(replica);
    API_END
}

int atm_batch_set_positions(atm_batch_t b, int replica, const double* pos) {
    API_BEGIN
    REQUIRE(b && pos, ATM_ERR_INVALID_ARGUMENT, "null argument");
    b->eng->set_positions(replica, pos);
    API_END
}

int atm_batch_set_parameter(atm_batch_t b, int replica, const char* name, double value) {
    API_BEGIN
    REQUIRE(b && name, ATM_ERR_INVALID_ARGUMENT, "null argument");
    int k = global_index(name);
    REQUIRE(k >= 0, ATM_ERR_INVALID_ARGUMENT, std::string("Called setParameter() with invalid parameter name: ") + name);
    b->eng->set_param(replica, k, value);
    API_END
}

int atm_batch_set_periodic_box_vectors(atm_batch_t b, int replica, const double* a, const double* b_, const double* c) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    double box[3], tilt[3];
    read_box(a, b_, c, box, tilt);
    b->eng->set_box(replica, box, tilt);
    API_END
}

int atm_batch_evaluate(atm_batch_t b, const double* pos_all, double* energies, double* forces, double* results) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    b->eng->evaluate_host(pos_all, energies, forces, nullptr, b->results.data(), b->matrix.data());
    if (results) std::memcpy(results, b->results.data(), sizeof(double) * b->results.size());
    b->evaluated = true;
    API_END
}

int atm_batch_evaluate_device(atm_batch_t b, const double* d_pos_all, double* d_forces, double* d_results,
                              void* stream) {
    API_BEGIN
    REQUIRE(b && d_pos_all, ATM_ERR_INVALID_ARGUMENT, "null argument");
    b->eng->evaluate_device(d_pos_all, d_forces, d_results, (cudaStream_t)stream);
    API_END
}

int atm_batch_set_displacements(atm_batch_t b, int replica, const double* displ) {
    API_BEGIN
    REQUIRE(b && displ, ATM_ERR_INVALID_ARGUMENT, "null argument");
    b->eng->set_displacements(replica, displ);
    API_END
}

int atm_batch_set_nonbonded_parameters(atm_batch_t b, int replica, const double* charge, const double* sigma,
                                       const double* epsilon) {
    API_BEGIN
    REQUIRE(b && charge && sigma && epsilon, ATM_ERR_INVALID_ARGUMENT, "null argument");
    b->eng->set_nonbonded_params(replica, charge, sigma, epsilon);
    API_END
}

int atm_batch_backward_device(atm_batch_t b, const double* d_g, double* d_dx, double* d_dd, double* d_dq,
                              double* d_dsig, double* d_deps, double* d_dparams, void* stream) {
    API_BEGIN
    REQUIRE(b && d_g, ATM_ERR_INVALID_ARGUMENT, "null argument");
    b->eng->backward(d_g, d_dx, d_dd, d_dq, d_dsig, d_deps, d_dparams, (cudaStream_t)stream);
    API_END
}

int atm_batch_backward(atm_batch_t b, const double* g, double* dx, double* dd, double* dq, double* dsig,
                       double* deps, double* dparams) {
    API_BEGIN
    REQUIRE(b && g, ATM_ERR_INVALID_ARGUMENT, "null argument");
    const int R = b->eng->replicas(), n = b->eng->total_atoms();
    // device staging, kept by the batch across calls
    const size_t need = (size_t)R + 3 * (size_t)n * 2 + 3 * (size_t)n + 5 * (size_t)R;
    if (b->scratch_n < need) {
        if (b->scratch) cudaFree(b->scratch);
        b->scratch = nullptr;
        if (cudaMalloc(&b->scratch, need * sizeof(double)) != cudaSuccess) throw Error(ATM_ERR_CUDA, "cudaMalloc");
        b->scratch_n = need;
    }
    double* dg = b->scratch;
    double* ddx = dg + R;
    double* ddd = ddx + 3 * (size_t)n;
    double* ddq = ddd + 3 * (size_t)n;
    double* dds = ddq + n;
    double* dde = dds + n;
    double* ddp = dde + n;
    if (cudaMemcpy(dg, g, sizeof(double) * R, cudaMemcpyHostToDevice) != cudaSuccess)
        throw Error(ATM_ERR_CUDA, "cudaMemcpy");
    const bool adj = b->eng->adjoint();
    b->eng->backward(dg, ddx, ddd, adj ? ddq : nullptr, adj ? dds : nullptr, adj ? dde : nullptr, ddp, 0);
    auto get = [](double* h, const double* d, size_t k) {
        if (h && cudaMemcpy(h, d, k * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
            throw Error(ATM_ERR_CUDA, "cudaMemcpy");
    };
    get(dx, ddx, 3 * (size_t)n);
    get(dd, ddd, 3 * (size_t)n);
    if (adj) {
        get(dq, ddq, n);
        get(dsig, dds, n);
        get(deps, dde, n);
    } else if (dq || dsig || deps) {
        throw Error(ATM_ERR_STATE, "Charge/sigma/epsilon gradients need a batch created with Adjoint=1");
    }
    get(dparams, ddp, 5 * (size_t)R);
    API_END
}

int atm_batch_get_list_info(atm_batch_t b, double* skin, long long* evaluations, long long* builds) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    if (skin) *skin = b->eng->list_skin();
    b->eng->list_counts(evaluations, builds);
    API_END
}

int atm_batch_energy_matrix(atm_batch_t b, double beta, double* matrix) {
    API_BEGIN
    REQUIRE(b && matrix, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(b->evaluated, ATM_ERR_STATE, "No evaluation has been run");
    for (size_t k = 0; k < b->matrix.size(); k++) matrix[k] = beta * b->matrix[k];
    API_END
}

int atm_batch_autotune(atm_batch_t b, int trials, int use_cache, char* report, size_t cap, size_t* len) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    REQUIRE(trials > 0, ATM_ERR_INVALID_ARGUMENT, "trials must be positive");
    std::string rep = b->eng->autotune(trials, use_cache != 0);
    copy_string(rep, report, cap, len);
    API_END
}

int atm_batch_set_profiling(atm_batch_t b, int on) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    b->eng->set_profiling(on != 0);
    API_END
}

int atm_batch_get_kernel_times(atm_batch_t b, char* names, size_t names_cap, double* ms, int cap, int* n) {
    API_BEGIN
    REQUIRE(b && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    const auto& t = b->eng->kernel_times();
    *n = (int)t.size();
    std::string joined;
    for (size_t k = 0; k < t.size(); k++) {
        if (k) joined += ",";
        joined += t[k].name;
        if (ms && (int)k < cap) ms[k] = t[k].ms;
    }
    copy_string(joined, names, names_cap, nullptr);
    API_END
}

int atm_batch_get_launch_count(atm_batch_t b, int* n) {
    API_BEGIN
    REQUIRE(b && n, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n = b->eng->launches_per_eval();
    API_END
}

int atm_batch_get_stats(atm_batch_t b, int* tiles, int* rows, int* max_row) {
    API_BEGIN
    REQUIRE(b, ATM_ERR_INVALID_ARGUMENT, "null batch");
    b->eng->stats(tiles, rows, max_row);
    API_END
}

// ---- MD ---------------------------------------------------------------------

int atm_md_create(const atm_system_t* systems, int n_replicas, int device, const char* properties,
                  double temperature, double friction, double step_size, unsigned long long seed, atm_md_t* out) {
    API_BEGIN
    REQUIRE(systems && out && n_replicas > 0, ATM_ERR_INVALID_ARGUMENT, "bad argument");
    REQUIRE(step_size > 0.0 && friction >= 0.0 && temperature >= 0.0, ATM_ERR_INVALID_ARGUMENT,
            "Invalid integrator parameters");
    auto props = parse_props(properties);
    bool diff = prop_bool(props, "DifferencePath", true);
    MdOptions opt;
    opt.temperature = temperature;
    opt.friction = friction;
    opt.step_size = step_size;
    opt.seed = seed;
    auto it = props.find("ReorderInterval");
    if (it != props.end()) opt.reorder_interval = std::stoi(it->second);
    it = props.find("ListSkin");
    if (it != props.end()) {
        if (it->second == "auto") {
            opt.list_skin = -1.0;
        } else {
            opt.list_skin = prop_double(props, "ListSkin", 0.1);
            REQUIRE(opt.list_skin >= 0.0, ATM_ERR_INVALID_ARGUMENT, "ListSkin must be a non-negative length or auto");
        }
    }
    it = props.find("CheckInterval");
    if (it != props.end()) opt.check_interval = std::stoi(it->second);
    it = props.find("TestFailListCheck");
    if (it != props.end()) opt.fail_check = std::stoi(it->second);
    std::vector<const System*> v;
    for (int r = 0; r < n_replicas; r++) {
        REQUIRE(systems[r], ATM_ERR_INVALID_ARGUMENT, "null system");
        v.push_back(&systems[r]->sys);
    }
    std::unique_ptr<atm_md_s> m(new atm_md_s);
    m->md.reset(new MDDriver(v, device, !diff, opt));
    m->md->engine().set_fused(prop_bool(props, "FusedTiles", false));
    m->md->engine().set_spread_owner(prop_bool(props, "SpreadByOwner", true));
    apply_spread_brick(m->md->engine(), props);
    *out = m.release();
    API_END
}

int atm_md_destroy(atm_md_t md) {
    API_BEGIN
    delete md;
    API_END
}

int atm_md_autotune(atm_md_t md, int trials, char* report, size_t cap, size_t* len) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null simulation");
    std::string rep = md->md->autotune(trials);
    copy_string(rep, report, cap, len);
    API_END
}

int atm_md_get_list_info(atm_md_t md, double* skin, long long* evaluations, long long* builds, int* redos) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null simulation");
    if (skin) *skin = md->md->engine().list_skin();
    if (redos) *redos = md->md->redos();
    md->md->engine().list_counts(evaluations, builds);
    API_END
}

int atm_md_get_num_particles(atm_md_t md, int* n_total) {
    API_BEGIN
    REQUIRE(md && n_total, ATM_ERR_INVALID_ARGUMENT, "null argument");
    *n_total = md->md->total_atoms();
    API_END
}

int atm_md_set_positions(atm_md_t md, const double* pos) {
    API_BEGIN
    REQUIRE(md && pos, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->set_positions(pos);
    API_END
}

int atm_md_set_velocities(atm_md_t md, const double* vel) {
    API_BEGIN
    REQUIRE(md && vel, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->set_velocities(vel);
    API_END
}

int atm_md_set_velocities_to_temperature(atm_md_t md, double temperature, unsigned long long seed) {
    API_BEGIN
    REQUIRE(md && temperature >= 0.0, ATM_ERR_INVALID_ARGUMENT, "bad argument");
    md->md->set_velocities_to_temperature(temperature, seed);
    API_END
}

int atm_md_set_parameter(atm_md_t md, int replica, const char* name, double value) {
    API_BEGIN
    REQUIRE(md && name, ATM_ERR_INVALID_ARGUMENT, "null argument");
    REQUIRE(replica >= 0 && replica < md->md->replicas(), ATM_ERR_INDEX, "Replica index out of range");
    int w = global_index(name);
    REQUIRE(w >= 0, ATM_ERR_INVALID_ARGUMENT, std::string("Unknown parameter: ") + name);
    md->md->set_param(replica, w, value);
    API_END
}

int atm_md_set_integrator(atm_md_t md, double temperature, double friction, double step_size) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->set_integrator(temperature, friction, step_size);
    API_END
}

int atm_md_step(atm_md_t md, int steps) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->step(steps);
    API_END
}

int atm_md_get_state(atm_md_t md, double* pos, double* vel, double* forces, double* potential, double* kinetic,
                     double* results) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->get_state(pos, vel, forces, potential, kinetic, results);
    API_END
}

int atm_md_set_recording(atm_md_t md, int interval, int capacity) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null argument");
    md->md->set_recording(interval, capacity);
    API_END
}

int atm_md_get_records(atm_md_t md, long long* steps, double* results, double* matrices, int max_records,
                       int* n_records) {
    API_BEGIN
    REQUIRE(md && n_records && max_records >= 0, ATM_ERR_INVALID_ARGUMENT, "bad argument");
    *n_records = md->md->get_records(steps, results, matrices, max_records);
    API_END
}

int atm_md_get_info(atm_md_t md, long long* steps, int* reorders, int* dof) {
    API_BEGIN
    REQUIRE(md, ATM_ERR_INVALID_ARGUMENT, "null argument");
    if (steps) *steps = md->md->step_count();
    if (reorders) *reorders = md->md->reorders();
    if (dof) {
        const auto& d = md->md->degrees_of_freedom();
        for (size_t r = 0; r < d.size(); r++) dof[r] = d[r];
    }
    API_END
}

}  // extern "C"
