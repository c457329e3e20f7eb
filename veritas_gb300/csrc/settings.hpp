// Host-side configuration, mirroring the reference's Input / Particles / Output structs
// and Settings class (Settings.hpp:4-67, Settings.cpp:5-195).  The user hooks the
// reference expects in its problem file (veritas.cpp: settingsOverride,
// InitialDistribution, GetBY/GetBZ, RefinementOverride) are virtual methods of
// vx::Problem; vx::LaserSlab is the built-in synthetic laser / plasma-slab problem.
#pragma once
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "vx_common.hpp"

namespace vx {

struct Input {  // Settings.hpp:4-11
    double minEfficiency = 0.6, dx = 0.5, k = 0.01;
    double refinementCriteria = 1e-8, cfl = 0.9, sizeWeight = 0.0;
    double preLength = 2, postLength = 2;
    unsigned int nx = 76 * 4, r = 2, Lfinest = 5;
    double plasma_xl_bound = 3.0e-6, plasma_xr_bound = 7.0e-6;
    std::vector<double> tempEM = {0.0};
};

struct Particles {  // Settings.hpp:13-20
    std::vector<double> mass = {9.10938291e-31};
    std::vector<double> charge = {-1.60217657e-19};
    std::vector<std::vector<double>> misc = {{0.0, 0.01}};
    std::vector<unsigned int> np = {50};
    std::vector<double> dp = {0.1};
    std::vector<double> pmin = {0.1};
};

struct Output {  // Settings.hpp:22-33 (file output itself is not part of the step)
    bool time = true, rectangleData = true, charge = true, energy = true, potential = true;
    bool EFieldLongitudinal = true, EFieldTransverse = true, BFieldTransverse = true, AFieldSquared = true;
    int precision = 15;
};

class Settings;

// The user's problem definition.  Default behaviour matches an empty override.
class Problem {
public:
    virtual ~Problem() = default;
    virtual void initialConditions(Input &grid, Particles &particles, Output &output) = 0;
    virtual void settingsOverride(Settings &s) = 0;
    virtual double InitialDistribution(const Settings &s, double x, double p, int particleType) const = 0;
    virtual double GetBY(const Settings &s, double x, double t) const = 0;
    virtual double GetBZ(const Settings &s, double x, double t) const = 0;
    virtual bool RefinementOverride(const Settings &s, double x, double p, int depth, int particleType) const = 0;
    virtual bool HasRefinementOverride() const { return true; }
    // Called at the end of the Settings constructor (derived sizes and fMax known).
    virtual void settingsComplete(const Settings &) {}
    // Optional: f(x, p) = density(x) * profile(p).  A problem that says so lets the FP32
    // form integrate the initial cell averages as a product of two 1-D quadratures.
    virtual bool Separable() const { return false; }
    virtual double Density(const Settings &, double, int) const { return 0.0; }
    virtual double Profile(const Settings &, double, int) const { return 0.0; }
    // Optional, exact product form: InitialDistribution(x, p) computes
    //   v = (X_0(x) * P_0(p)) / C_0;  v = v + (X_t(x) * P_t(p)) / C_t  (t = 1 .. terms-1)
    // in exactly these IEEE double operations.  A problem that says so (ProductTerms > 0)
    // has its FP64 quadrature formed on the device from the host-evaluated factors, with
    // the same bits as the host loop.
    virtual int ProductTerms(int) const { return 0; }
    virtual double XFactor(const Settings &, int, double, int) const { return 0.0; }
    virtual double PFactor(const Settings &, int, double, int) const { return 0.0; }
    virtual double Divisor(const Settings &, int, int) const { return 1.0; }
};

// Parameters of the built-in laser / plasma-slab problem (lengths in laser wavelengths,
// momenta in m_e c, temperatures in keV).  Field layout matches vx_problem in vx.h.
struct LaserSlabParams {
    double lambda = 1e-6;
    double L = 100.0;
    unsigned nx = 2048, np = 256, Lfinest = 1, r = 2;
    double pmax = 2.0;
    double dens = 0.01;
    double x1 = 15, x2 = 20, x3 = 80, x4 = 85;
    double Te = 1.0;
    double p0 = 0.0;
    double pert_amp = 0.0, pert_k = 1.0;
    double a0 = 1.0, fwhm = 10.0, delay = 10.0;
    double cfl = 0.5, minEff = 0.75, crit = 1e-6, sizeWeight = 1.0;
    int quadDepth = 2;
    double bdens = 0.0, bp0 = 0.0, bTe = 1.0;  // beam population: density fraction, drift, keV
    // mobile ions (second species) when mi > 0: charge +e, mass mi m_e, the electrons'
    // density profile, temperature iTe [keV], p in [-ipmax, ipmax] m_i c
    double mi = 0.0, iTe = 1.0, ipmax = 0.1;
};

class LaserSlab : public Problem {
public:
    explicit LaserSlab(const LaserSlabParams &p) : P(p) {}
    void initialConditions(Input &grid, Particles &particles, Output &output) override;
    void settingsOverride(Settings &s) override;
    double InitialDistribution(const Settings &s, double x, double p, int particleType) const override;
    double GetBY(const Settings &s, double x, double t) const override;
    double GetBZ(const Settings &s, double x, double t) const override;
    bool RefinementOverride(const Settings &s, double x, double p, int depth, int particleType) const override {
        return false;
    }
    bool HasRefinementOverride() const override { return false; }
    bool Separable() const override { return true; }
    double Density(const Settings &s, double x, int particleType) const override;
    double Profile(const Settings &s, double p, int particleType) const override;
    int ProductTerms(int particleType) const override { return (P.bdens != 0.0 && particleType == 0) ? 2 : 1; }
    double XFactor(const Settings &s, int term, double x, int particleType) const override;
    double PFactor(const Settings &s, int term, double p, int particleType) const override;
    double Divisor(const Settings &s, int term, int particleType) const override;
    double slab_density(double xl) const;
    LaserSlabParams P;
    double beam_T = 0.0, beam_p = 0.0;  // beam temperature [J] and drift [kg m/s]
};

class Settings {  // Settings.hpp:35-65
public:
    Output output;
    double dx, time, minEfficiency, preLength, postLength, refinementCriteria, cfl, sizeWeight, plasma_xl_bound,
        plasma_xr_bound;
    std::vector<double> m, q, m_inv, dp, fMax, tempEM, pmin;
    std::vector<std::vector<double>> temp;
    unsigned int x_size_finest, x_size, refinementRatio;
    int maxDepth, quadratureDepth = 0;
    std::vector<unsigned int> p_size, p_size_finest;
    std::shared_ptr<Problem> problem;

    // Throws std::invalid_argument where the reference exits (Settings.cpp:35-50).
    Settings(const Input &grid, const Particles &particles, const Output &out, std::shared_ptr<Problem> problem);
    double InitialDistribution(double x, double p, int particleType) const {
        return problem->InitialDistribution(*this, x, p, particleType);
    }
    double GetDp(int level, int particleType) const;
    double GetDx(int level) const;
    int GetXSize(int level) const;
    int GetPSize(int level, int particleType) const;
    double GetMass(int i) const { return m.at(i); }
    double GetCharge(int i) const { return q.at(i); }
    double GetfMax(int i) const { return fMax.at(i); }
    void UpdateTime(int step, double dt);
    double GetBY(double x, double t) const { return problem->GetBY(*this, x, t); }
    double GetBZ(double x, double t) const { return problem->GetBZ(*this, x, t); }
    void DetermineMaximum();
    bool RefinementOverride(double x, double p, int depth, int particleType) const {
        return problem->RefinementOverride(*this, x, p, depth, particleType);
    }
};

}  // namespace vx
