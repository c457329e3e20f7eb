#include "settings.hpp"

#include <stdexcept>

namespace vx {

static const double kMe = 9.10938291e-31;
static const double kQe = -1.60217657e-19;
static const double kKeV = 1.602176565e-16;

Settings::Settings(const Input &grid, const Particles &particles, const Output &out, std::shared_ptr<Problem> prob)
    : problem(std::move(prob)) {
    // Settings.cpp:5-54
    output = out;
    dx = grid.dx;
    dp = particles.dp;
    maxDepth = (int)grid.Lfinest - 1;
    x_size = grid.nx;
    p_size = particles.np;
    refinementRatio = grid.r;
    refinementCriteria = grid.refinementCriteria;
    minEfficiency = grid.minEfficiency;
    time = 0.0;
    preLength = grid.preLength;
    postLength = grid.postLength;
    cfl = grid.cfl;
    sizeWeight = grid.sizeWeight;
    m = particles.mass;
    q = particles.charge;
    tempEM = grid.tempEM;
    temp = particles.misc;
    pmin = particles.pmin;
    plasma_xl_bound = grid.plasma_xl_bound;
    plasma_xr_bound = grid.plasma_xr_bound;
    problem->settingsOverride(*this);
    if (refinementRatio % 2)
        throw std::invalid_argument("Mesh refinement ratio 'refinementRatio' must be an even value.");
    if (x_size % refinementRatio != 0)
        throw std::invalid_argument("'x_size' must be completely divisible by the Mesh refinement ratio.");
    for (unsigned int p = 0; p < p_size.size(); p++)
        if (p_size[p] % refinementRatio != 0)
            throw std::invalid_argument("'p_size' must be completely divisible by the Mesh refinement ratio.");
    if (maxDepth < 0) throw std::invalid_argument("Lfinest must be at least 1.");
    x_size_finest = x_size * std::pow(refinementRatio, maxDepth);
    for (unsigned int i = 0; i < p_size.size(); i++) p_size_finest.push_back(p_size[i] * std::pow(refinementRatio, maxDepth));
    for (double mm : m) m_inv.push_back(1 / mm);
    fMax.resize(q.size(), 0.0);
    DetermineMaximum();
    problem->settingsComplete(*this);
}

double Settings::GetDp(int level, int particleType) const {
    return std::pow(refinementRatio, level - maxDepth) * dp.at(particleType);
}
double Settings::GetDx(int level) const { return std::pow(refinementRatio, level - maxDepth) * dx; }
int Settings::GetXSize(int level) const { return x_size * std::pow(refinementRatio, -level + maxDepth); }
int Settings::GetPSize(int level, int particleType) const {
    return p_size[particleType] * std::pow(refinementRatio, -level + maxDepth);
}

void Settings::UpdateTime(int step, double dt) {  // Settings.cpp:166-179
    if (step == 1) time += (0.5 * dt);
    else if (step == 2) time += (0.332 - 0.5) * dt;
    else if (step == 3) time += (0.62 - 0.332) * dt;
    else if (step == 4) time += (0.85 - 0.62) * dt;
    else if (step == 5) time += (1.0 - 0.85) * dt;
}

void Settings::DetermineMaximum() {  // Settings.cpp:181-194 (mValue carried across species)
    double dx0 = GetDx(0);
    double mValue(0.0);
    for (unsigned int j = 0; j < q.size(); j++) {
        for (int i = 0; i < GetXSize(0); i++) {
            double t = InitialDistribution((i + 0.5) * dx0, 0, j);
            mValue = t > mValue ? t : mValue;
        }
        fMax[j] = mValue;
    }
}

// ---------------------------------------------------------------- LaserSlab
void LaserSlab::initialConditions(Input &grid, Particles &particles, Output &output) {
    grid.minEfficiency = P.minEff;
    grid.dx = 1.0;
    grid.refinementCriteria = P.crit;
    grid.cfl = P.cfl;
    grid.sizeWeight = P.sizeWeight;
    grid.preLength = 0;
    grid.postLength = 0;
    grid.nx = P.nx;
    grid.r = P.r;
    grid.Lfinest = P.Lfinest;
    grid.tempEM = {0.0};
    particles.mass = {kMe};
    particles.charge = {kQe};
    particles.misc = {{0.0, 0.0}};
    particles.np = {P.np};
    particles.dp = {0.1};
    particles.pmin = {0.0};
    if (P.mi > 0.0) {  // mobile ions
        particles.mass.push_back(P.mi * kMe);
        particles.charge.push_back(-kQe);
        particles.misc.push_back({0.0, 0.0});
        particles.np.push_back(P.np);
        particles.dp.push_back(0.1);
        particles.pmin.push_back(0.0);
    }
    output = Output();
}

void LaserSlab::settingsOverride(Settings &s) {
    double mc = s.m[0] * kCs;
    s.dp[0] = 2.0 * P.pmax * mc / s.p_size[0];
    s.pmin[0] = -P.pmax * mc;
    s.dx = P.L * P.lambda / s.x_size;
    s.quadratureDepth = P.quadDepth;
    double T = P.lambda / kCs;
    double omega = kDPI / T;
    double Nc = omega * omega * s.m[0] * kEps0 / (s.q[0] * s.q[0]);
    s.temp[0].resize(3, 0.0);
    s.temp[0][0] = P.dens * Nc;
    s.temp[0][1] = s.m[0] * (P.Te * kKeV);
    s.temp[0][2] = P.p0 * mc;
    s.tempEM.resize(2, 0.0);
    s.tempEM[0] = P.lambda;
    s.tempEM[1] = P.a0 * mc / std::fabs(s.q[0]);
    beam_T = s.m[0] * (P.bTe * kKeV);
    beam_p = P.bp0 * mc;
    if (s.m.size() > 1) {  // ions: same density, own temperature and momentum range
        double mci = s.m[1] * kCs;
        s.dp[1] = 2.0 * P.ipmax * mci / s.p_size[1];
        s.pmin[1] = -P.ipmax * mci;
        s.temp[1].resize(3, 0.0);
        s.temp[1][0] = P.dens * Nc;
        s.temp[1][1] = s.m[1] * (P.iTe * kKeV);
        s.temp[1][2] = 0.0;
    }
}

double LaserSlab::slab_density(double xl) const {
    double s;
    if (xl <= P.x1 || xl >= P.x4) s = 0.0;
    else if (xl < P.x2) s = (xl - P.x1) / (P.x2 - P.x1);
    else if (xl <= P.x3) s = 1.0;
    else s = (P.x4 - xl) / (P.x4 - P.x3);
    if (P.pert_amp != 0.0) s = s * (1.0 + P.pert_amp * std::sin(kDPI * P.pert_k * xl / P.L));
    return s;
}

double LaserSlab::InitialDistribution(const Settings &s, double x, double p, int particleType) const {
    double ne = s.temp[particleType][0] * slab_density(x / P.lambda);
    double dpv = p - s.temp[particleType][2];
    double v = ne * std::exp(-(dpv * dpv) / (2.0 * s.temp[particleType][1])) / std::sqrt(kDPI * s.temp[particleType][1]);
    if (P.bdens != 0.0 && particleType == 0) {  // drifting electron population, own temperature
        double dbv = p - beam_p;
        v += P.bdens * ne * std::exp(-(dbv * dbv) / (2.0 * beam_T)) / std::sqrt(kDPI * beam_T);
    }
    return v;
}

// InitialDistribution's terms: (ne * exp) / sqrt for the plasma, ((bdens * ne) * exp) /
// sqrt for the electron beam (the operations of InitialDistribution above).
double LaserSlab::XFactor(const Settings &s, int term, double x, int particleType) const {
    double ne = s.temp[particleType][0] * slab_density(x / P.lambda);
    return term == 0 ? ne : P.bdens * ne;
}

double LaserSlab::PFactor(const Settings &s, int term, double p, int particleType) const {
    if (term == 0) {
        double dpv = p - s.temp[particleType][2];
        return std::exp(-(dpv * dpv) / (2.0 * s.temp[particleType][1]));
    }
    double dbv = p - beam_p;
    return std::exp(-(dbv * dbv) / (2.0 * beam_T));
}

double LaserSlab::Divisor(const Settings &s, int term, int particleType) const {
    return term == 0 ? std::sqrt(kDPI * s.temp[particleType][1]) : std::sqrt(kDPI * beam_T);
}

double LaserSlab::Density(const Settings &s, double x, int particleType) const {
    return s.temp[particleType][0] * slab_density(x / P.lambda);
}

double LaserSlab::Profile(const Settings &s, double p, int particleType) const {
    double dpv = p - s.temp[particleType][2];
    double v = std::exp(-(dpv * dpv) / (2.0 * s.temp[particleType][1])) / std::sqrt(kDPI * s.temp[particleType][1]);
    if (P.bdens != 0.0 && particleType == 0) {
        double dbv = p - beam_p;
        v += P.bdens * std::exp(-(dbv * dbv) / (2.0 * beam_T)) / std::sqrt(kDPI * beam_T);
    }
    return v;
}

double LaserSlab::GetBY(const Settings &s, double x, double t) const { return 0.0; }

// Linearly polarised pulse A_y = A0 g(t - x/c) cos(w t - k x) with a Gaussian field
// envelope g; returns B_z = dA_y/dx.
double LaserSlab::GetBZ(const Settings &s, double x, double t) const {
    double T = s.tempEM[0] / kCs;
    double k = kDPI / s.tempEM[0];
    double omega = kCs * k;
    double F = P.fwhm * T;
    double tau = (t - x / kCs) - P.delay * T;
    double c4 = 4.0 * std::log(2.0) / (F * F);
    double g = std::exp(-c4 * tau * tau);
    double gp = -2.0 * c4 * tau * g;
    double ph = omega * t - k * x;
    return s.tempEM[1] * (k * g * std::sin(ph) - (gp / kCs) * std::cos(ph));
}

}  // namespace vx
