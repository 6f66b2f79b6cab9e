// Host object model of the ATM path: ATMMetaForce (same members and semantics as
// the reference's openmmapi/include/ATMMetaForce.h:54-335), the inner
// NonbondedForce description, and a System that owns them.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace atm {

// Error carrying one of the ATM_* status codes of include/atm_capi.h.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum GlobalIndex { LAMBDA1 = 0, LAMBDA2, ALPHA, U0, W0, UMAX, UBCORE, ACORE, DIRECTION, NUM_GLOBALS };

// Global-parameter names, ATMMetaForce.h:151-218.
const char* global_name(int which);
int global_index(const std::string& name);  // -1 if unknown
extern const char* const kVersion;          // ATMMetaForceVersion.h:4

class ATMMetaForce {
public:
    struct ParticleInfo {  // ATMMetaForce.h:321-334
        int particle = -1;
        double dx = 0, dy = 0, dz = 0;
    };
    ATMMetaForce(double lambda1, double lambda2, double alpha, double u0, double w0, double umax, double ubcore,
                 double acore, double direction, const std::vector<int>& groups);
    int addParticle(int particle, double dx, double dy, double dz);
    void getParticleParameters(int index, int& particle, double& dx, double& dy, double& dz) const;
    void setParticleParameters(int index, int particle, double dx, double dy, double dz);
    int getNumParticles() const { return (int)particles.size(); }
    double getDefault(int which) const { return defaults[which]; }
    const std::vector<int>& getVariableForceGroups() const { return groups; }
    int getForceGroup() const { return forceGroup; }
    void setForceGroup(int g);
    const std::string& getName() const { return name; }
    void setName(const std::string& n) { name = n; }

    double defaults[NUM_GLOBALS];
    std::vector<int> groups;
    std::vector<ParticleInfo> particles;
    int forceGroup = 0;
    std::string name = "ATMMetaForce";
};

struct Exception {
    int i, j;
    double qq, sig, eps;
};

class NonbondedForce {
public:
    enum Method { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2, PME = 4 };
    int addParticle(double q, double sig, double eps);
    int addException(int i, int j, double qq, double sig, double eps);
    std::vector<double> charge, sigma, epsilon;
    std::vector<Exception> exceptions;
    int method = NoCutoff;
    double cutoff = 1.0;
    double epsRF = 78.3;       // OpenMM's default reaction-field dielectric
    double ewaldTol = 5e-4;    // OpenMM's default Ewald error tolerance
    double alpha = 0.0;        // 0: derive from the tolerance
    int grid[3] = {0, 0, 0};
    bool dispersionCorrection = true;  // OpenMM's default
    int forceGroup = 0;
};

// Terms integrated alongside the ATM force by the MD driver (force group 0 of
// the reference's test and examples: python/tests/test_abfe.py:101-103).
struct Bond {  // OpenMM HarmonicBondForce: (k/2)(r - length)^2, no periodic image
    int i, j;
    double length, k;
};
struct Angle {  // OpenMM HarmonicAngleForce: (k/2)(theta - angle)^2 at vertex j
    int i, j, l;
    double angle, k;
};
struct Constraint {  // System::addConstraint: fixed distance between two particles
    int i, j;
    double distance;
};
// Flat-bottom harmonic restraint between the mass-weighted centroids of two
// particle groups: (kf/2) step(d - tol) (d - tol)^2, d = |c1 - offset - c2|, no
// periodic image (python/ATMMetaForceUtils.py:79-138, addVsiteRestraintForceCMCM).
struct CentroidRestraint {
    std::vector<int> g1, g2;
    double kf, tol;
    double offset[3];
};
// Flat-bottom harmonic position restraint: 0.5 fc step(d - tol)(d - tol)^2 with
// d the (periodic) distance to (x0, y0, z0) (python/ATMMetaForceUtils.py:707-752).
struct PositionRestraint {
    int particle;
    double x0, y0, z0, fc, tol;
};

class System {
public:
    int addParticle(double m) {
        masses.push_back(m);
        return (int)masses.size() - 1;
    }
    std::vector<double> masses;
    double box[3] = {2.0, 2.0, 2.0};  // OpenMM's default box (diagonal of the box vectors)
    double tilt[3] = {0.0, 0.0, 0.0}; // b_x, c_x, c_y of reduced triclinic box vectors
    std::unique_ptr<NonbondedForce> nonbonded;
    std::unique_ptr<ATMMetaForce> atm;
    std::vector<Bond> bonds;
    std::vector<Angle> angles;
    std::vector<Constraint> constraints;
    std::vector<CentroidRestraint> centroid_restraints;
    std::vector<PositionRestraint> position_restraints;
    bool position_restraints_periodic = true;
};

// XML of serialization/src/ATMMetaForceProxy.cpp:11-79 inside OpenMM's
// <Force type="ATMMetaForce" ...> wrapper.
std::string serialize(const ATMMetaForce& f);
std::unique_ptr<ATMMetaForce> deserialize(const std::string& xml);

// OpenMM's documented PME parameter rule (alpha from the tolerance, grid from
// the box), without rounding to FFT-friendly sizes, as the Reference platform.
void pme_parameters(double cutoff, double tol, const double* box, double& alpha, int* grid);

}  // namespace atm
