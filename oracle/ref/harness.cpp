// ORACLE / TEST INFRASTRUCTURE — problem definition and driver for the *reference*
// Veritas build (the unmodified sources under the reference tree, compiled by
// oracle/ref/build_ref.sh).  This translation unit plays the role of the reference's
// user file veritas.cpp (veritas.cpp:7-170): it supplies the Settings hooks the user is
// expected to write (settingsOverride, InitialDistribution, GetBY/GetBZ,
// RefinementOverride) for the synthetic laser/slab problem, plus a main() that steps
// the solver and dumps binary state snapshots for parity tests.
//
// Private state of SolverManager / EMFieldSolver / Rectangle is read through the
// explicit-instantiation member-pointer idiom (legal C++: explicit instantiation may
// name private members), so the reference sources stay untouched.
#include "veritas.hpp"
#include "Settings.hpp"
#include "SolverManager.hpp"
#include "EMSolver.hpp"
#include "Mesh.hpp"
#include "Level.hpp"
#include "Rectangle.hpp"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

// ---------------------------------------------------------------- private access
template <class Tag>
struct Stolen {
    static typename Tag::type ptr;
};
template <class Tag>
typename Tag::type Stolen<Tag>::ptr;
template <class Tag, typename Tag::type M>
struct Rob {
    struct Filler {
        Filler() { Stolen<Tag>::ptr = M; }
    };
    static Filler filler;
};
template <class Tag, typename Tag::type M>
typename Rob<Tag, M>::Filler Rob<Tag, M>::filler;

#define VX_ROB(NAME, CLASS, TYPE, MEMBER)                 \
    struct NAME {                                         \
        typedef TYPE CLASS::*type;                        \
    };                                                    \
    template struct Rob<NAME, &CLASS::MEMBER>;
#define VX_GET(OBJ, NAME) ((OBJ).*Stolen<NAME>::ptr)

VX_ROB(SM_meshes, SolverManager, std::vector<std::shared_ptr<Mesh>>, meshes)
VX_ROB(SM_em, SolverManager, std::shared_ptr<EMFieldSolver>, EMSolver)
VX_ROB(EM_pre, EMFieldSolver, int, n_prepad)
VX_ROB(EM_post, EMFieldSolver, int, n_postpad)
VX_ROB(EM_xsize, EMFieldSolver, unsigned int, x_size)
VX_ROB(EM_charge, EMFieldSolver, std::vector<double>, charge)
VX_ROB(EM_J, EMFieldSolver, std::vector<double>, J)
VX_ROB(EM_By, EMFieldSolver, std::vector<double>, By)
VX_ROB(EM_Bz, EMFieldSolver, std::vector<double>, Bz)
VX_ROB(EM_Ey, EMFieldSolver, std::vector<double>, Ey)
VX_ROB(EM_Ez, EMFieldSolver, std::vector<double>, Ez)
VX_ROB(EM_Ay, EMFieldSolver, std::vector<double>, Ay)
VX_ROB(EM_Az, EMFieldSolver, std::vector<double>, Az)
VX_ROB(EM_asq, EMFieldSolver, std::vector<double>, a_squared)
VX_ROB(EM_neut, EMFieldSolver, std::vector<double>, neutralizationCharge)
VX_ROB(EM_phi, EMFieldSolver, double *, PHI)
VX_ROB(EM_ex0, EMFieldSolver, double, Ex0)
VX_ROB(R_depth, Rectangle, int, depth)
VX_ROB(R_up, Rectangle, bool, up)
VX_ROB(R_down, Rectangle, bool, down)
VX_ROB(R_left, Rectangle, bool, left)
VX_ROB(R_right, Rectangle, bool, right)

#ifndef VX_HOOKS_PROBLEM
// ---------------------------------------------------------------- problem parameters
// Synthetic laser / plasma-slab problem (all lengths in laser wavelengths, momenta in
// m_e c, temperatures in keV).  The product carries its own copy of these formulas.
struct Problem {
    double lambda = 1e-6;
    double L = 100.0;                                // domain length [lambda]
    unsigned nx = 2048, np = 256, Lfinest = 1, r = 2;
    double pmax = 2.0;                               // p in [-pmax, pmax] m_e c
    double dens = 0.01;                              // plateau density / n_c
    double x1 = 15, x2 = 20, x3 = 80, x4 = 85;      // ramp up [x1,x2], plateau, ramp down [x3,x4]
    double Te = 1.0;                                 // keV
    double p0 = 0.0;                                 // drift [m_e c]
    double bdens = 0.0, bp0 = 0.0, bTe = 1.0;        // beam population: density fraction, drift, keV
    double pert_amp = 0.0, pert_k = 1.0;             // density modulation
    double a0 = 1.0, fwhm = 10.0, delay = 10.0;      // laser [periods]
    double cfl = 0.5, minEff = 0.75, crit = 1e-6, sizeWeight = 1.0;
    int quadDepth = 2;
    double mi = 0.0, iTe = 1.0, ipmax = 0.1;          // mobile ions when mi > 0 (mass / m_e, keV, m_i c)
    bool diag = false;                               // enable the reference's text outputs
};
static Problem P;
static double beam_T = 0.0, beam_p = 0.0;

static const double kMe = 9.10938291e-31;
static const double kQe = -1.60217657e-19;
static const double kKeV = 1.602176565e-16;

static double slab_density(double xl) {
    // xl in wavelengths
    double s;
    if (xl <= P.x1 || xl >= P.x4) s = 0.0;
    else if (xl < P.x2) s = (xl - P.x1) / (P.x2 - P.x1);
    else if (xl <= P.x3) s = 1.0;
    else s = (P.x4 - xl) / (P.x4 - P.x3);
    if (P.pert_amp != 0.0) s = s * (1.0 + P.pert_amp * std::sin(DPI * P.pert_k * xl / P.L));
    return s;
}

void initialConditions(Input &grid, Particles &particles, Output &output) {
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
    if (P.mi > 0.0) {  // mobile ions: second species
        particles.mass.push_back(P.mi * kMe);
        particles.charge.push_back(-kQe);
        particles.misc.push_back({0.0, 0.0});
        particles.np.push_back(P.np);
        particles.dp.push_back(0.1);
        particles.pmin.push_back(0.0);
    }
    // the reference's text outputs only in the diag_every mode
    output.time = output.rectangleData = output.charge = output.energy = output.potential = P.diag;
    output.EFieldLongitudinal = output.EFieldTransverse = output.BFieldTransverse = output.AFieldSquared = P.diag;
    output.precision = 15;
}

void Settings::settingsOverride() {
    double mc = m[0] * cs;
    dp[0] = 2.0 * P.pmax * mc / p_size[0];
    pmin[0] = -P.pmax * mc;
    dx = P.L * P.lambda / x_size;
    quadratureDepth = P.quadDepth;
    double T = P.lambda / cs;
    double omega = DPI / T;
    double Nc = omega * omega * m[0] * eps0 / (q[0] * q[0]);
    temp[0].resize(3, 0.0);
    temp[0][0] = P.dens * Nc;
    temp[0][1] = m[0] * (P.Te * kKeV);
    temp[0][2] = P.p0 * mc;
    tempEM.resize(2, 0.0);
    tempEM[0] = P.lambda;
    tempEM[1] = P.a0 * mc / std::fabs(q[0]);
    beam_T = m[0] * (P.bTe * kKeV);
    beam_p = P.bp0 * mc;
    if (m.size() > 1) {
        double mci = m[1] * cs;
        dp[1] = 2.0 * P.ipmax * mci / p_size[1];
        pmin[1] = -P.ipmax * mci;
        temp[1].resize(3, 0.0);
        temp[1][0] = P.dens * Nc;
        temp[1][1] = m[1] * (P.iTe * kKeV);
        temp[1][2] = 0.0;
    }
}

bool Settings::RefinementOverride(double x, double p, int depth, int particleType) {
    return false;
}

double Settings::GetBY(double x, double t) {
    return 0.0;
}

double Settings::GetBZ(double x, double t) {
    double T = tempEM[0] / cs;
    double k = DPI / tempEM[0];
    double omega = cs * k;
    double F = P.fwhm * T;
    double tau = (t - x / cs) - P.delay * T;
    double c4 = 4.0 * std::log(2.0) / (F * F);
    double g = std::exp(-c4 * tau * tau);
    double gp = -2.0 * c4 * tau * g;
    double ph = omega * t - k * x;
    return tempEM[1] * (k * g * std::sin(ph) - (gp / cs) * std::cos(ph));
}

double Settings::InitialDistribution(double x, double p, int particleType) {
    double ne = temp[particleType][0] * slab_density(x / P.lambda);
    double dpv = p - temp[particleType][2];
    double v = ne * std::exp(-(dpv * dpv) / (2.0 * temp[particleType][1])) / std::sqrt(DPI * temp[particleType][1]);
    if (P.bdens != 0.0 && particleType == 0) {  // drifting electron population
        double dbv = p - beam_p;
        v += P.bdens * ne * std::exp(-(dbv * dbv) / (2.0 * beam_T)) / std::sqrt(DPI * beam_T);
    }
    return v;
}

#else  // VX_HOOKS_PROBLEM
// ---------------------------------------------------------------- C-hook problem
// The reference's Settings hooks forwarded to a user problem written against the C
// structs of include/vx.h (tests/hooks/sin2_problem.c), so that the reference build and
// the GPU path (vx_run_create_hooks) run the same user code.  The hooks see the Settings
// as vx.h describes: taken after settingsOverride and refreshed once the Settings are
// complete (main, after the constructor).
#include "sin2_problem.h"

static sin2_params HP;
static vx_settings VIEW;

template <class V>
static void put_vec(const V &v, int32_t *n, double *out) {
    *n = (int32_t)v.size();
    for (size_t i = 0; i < v.size(); i++) out[i] = v[i];
}
static void settings_to_c(const Settings &s, vx_settings &c) {
    std::memset(&c, 0, sizeof c);
    c.dx = s.dx, c.time = s.time, c.minEfficiency = s.minEfficiency, c.preLength = s.preLength;
    c.postLength = s.postLength, c.refinementCriteria = s.refinementCriteria, c.cfl = s.cfl;
    c.sizeWeight = s.sizeWeight, c.plasma_xl_bound = s.plasma_xl_bound, c.plasma_xr_bound = s.plasma_xr_bound;
    c.nspecies = (int32_t)s.m.size();
    for (size_t i = 0; i < s.m.size(); i++) {
        c.m[i] = s.m[i];
        c.q[i] = s.q[i];
        c.m_inv[i] = i < s.m_inv.size() ? s.m_inv[i] : 0.0;
        c.dp[i] = s.dp[i];
        c.fMax[i] = i < s.fMax.size() ? s.fMax[i] : 0.0;
        c.pmin[i] = s.pmin[i];
        put_vec(s.temp[i], &c.ntemp[i], c.temp[i]);
        c.p_size[i] = s.p_size[i];
        c.p_size_finest[i] = i < s.p_size_finest.size() ? s.p_size_finest[i] : 0;
    }
    put_vec(s.tempEM, &c.ntempEM, c.tempEM);
    c.x_size_finest = s.x_size_finest, c.x_size = s.x_size, c.refinementRatio = s.refinementRatio;
    c.maxDepth = s.maxDepth, c.quadratureDepth = s.quadratureDepth;
}

void initialConditions(Input &grid, Particles &particles, Output &output) {
    vx_input g;
    vx_particles p;
    vx_output o;
    std::memset(&g, 0, sizeof g);
    std::memset(&p, 0, sizeof p);
    g.minEfficiency = grid.minEfficiency, g.dx = grid.dx, g.k = grid.k;
    g.refinementCriteria = grid.refinementCriteria, g.cfl = grid.cfl, g.sizeWeight = grid.sizeWeight;
    g.preLength = grid.preLength, g.postLength = grid.postLength;
    g.nx = grid.nx, g.r = grid.r, g.Lfinest = grid.Lfinest;
    g.plasma_xl_bound = grid.plasma_xl_bound, g.plasma_xr_bound = grid.plasma_xr_bound;
    put_vec(grid.tempEM, &g.ntempEM, g.tempEM);
    p.nspecies = (int32_t)particles.mass.size();
    for (int s = 0; s < p.nspecies; s++) {
        p.mass[s] = particles.mass[s], p.charge[s] = particles.charge[s], p.np[s] = particles.np[s];
        p.dp[s] = particles.dp[s], p.pmin[s] = particles.pmin[s];
        put_vec(particles.misc[s], &p.nmisc[s], p.misc[s]);
    }
    o.time = output.time, o.rectangleData = output.rectangleData, o.charge = output.charge;
    o.energy = output.energy, o.potential = output.potential, o.EFieldLongitudinal = output.EFieldLongitudinal;
    o.EFieldTransverse = output.EFieldTransverse, o.BFieldTransverse = output.BFieldTransverse;
    o.AFieldSquared = output.AFieldSquared, o.precision = output.precision;
    sin2_initial_conditions(&HP, &g, &p, &o);
    grid.minEfficiency = g.minEfficiency, grid.dx = g.dx, grid.k = g.k;
    grid.refinementCriteria = g.refinementCriteria, grid.cfl = g.cfl, grid.sizeWeight = g.sizeWeight;
    grid.preLength = g.preLength, grid.postLength = g.postLength;
    grid.nx = g.nx, grid.r = g.r, grid.Lfinest = g.Lfinest;
    grid.plasma_xl_bound = g.plasma_xl_bound, grid.plasma_xr_bound = g.plasma_xr_bound;
    grid.tempEM.assign(g.tempEM, g.tempEM + g.ntempEM);
    particles.mass.clear(), particles.charge.clear(), particles.np.clear();
    particles.dp.clear(), particles.pmin.clear(), particles.misc.clear();
    for (int s = 0; s < p.nspecies; s++) {
        particles.mass.push_back(p.mass[s]);
        particles.charge.push_back(p.charge[s]);
        particles.np.push_back(p.np[s]);
        particles.dp.push_back(p.dp[s]);
        particles.pmin.push_back(p.pmin[s]);
        particles.misc.push_back(std::vector<double>(p.misc[s], p.misc[s] + p.nmisc[s]));
    }
    output.time = o.time, output.rectangleData = o.rectangleData, output.charge = o.charge;
    output.energy = o.energy, output.potential = o.potential, output.EFieldLongitudinal = o.EFieldLongitudinal;
    output.EFieldTransverse = o.EFieldTransverse, output.BFieldTransverse = o.BFieldTransverse;
    output.AFieldSquared = o.AFieldSquared, output.precision = o.precision;
}

void Settings::settingsOverride() {
    settings_to_c(*this, VIEW);
    sin2_settings_override(&HP, &VIEW);
    dx = VIEW.dx, time = VIEW.time, minEfficiency = VIEW.minEfficiency, preLength = VIEW.preLength;
    postLength = VIEW.postLength, refinementCriteria = VIEW.refinementCriteria, cfl = VIEW.cfl;
    sizeWeight = VIEW.sizeWeight, plasma_xl_bound = VIEW.plasma_xl_bound, plasma_xr_bound = VIEW.plasma_xr_bound;
    for (int i = 0; i < VIEW.nspecies; i++) {
        m[i] = VIEW.m[i], q[i] = VIEW.q[i], dp[i] = VIEW.dp[i], pmin[i] = VIEW.pmin[i];
        temp[i].assign(VIEW.temp[i], VIEW.temp[i] + VIEW.ntemp[i]);
        p_size[i] = VIEW.p_size[i];
    }
    tempEM.assign(VIEW.tempEM, VIEW.tempEM + VIEW.ntempEM);
    x_size = VIEW.x_size, refinementRatio = VIEW.refinementRatio;
    maxDepth = VIEW.maxDepth, quadratureDepth = VIEW.quadratureDepth;
    settings_to_c(*this, VIEW);
}

bool Settings::RefinementOverride(double x, double p, int depth, int particleType) {
    return sin2_refinement_override(&HP, &VIEW, x, p, depth, particleType) != 0;
}

double Settings::GetBY(double x, double t) { return sin2_get_by(&HP, &VIEW, x, t); }

double Settings::GetBZ(double x, double t) { return sin2_get_bz(&HP, &VIEW, x, t); }

double Settings::InitialDistribution(double x, double p, int particleType) {
    return sin2_initial_distribution(&HP, &VIEW, x, p, particleType);
}
#endif  // VX_HOOKS_PROBLEM

bool LOUD = false, NOISY = false;

// ---------------------------------------------------------------- state dump
static void wr(FILE *fp, const void *p, size_t n) {
    if (n && fwrite(p, 1, n, fp) != n) {
        perror("fwrite");
        exit(2);
    }
}
static void wi(FILE *fp, long long v) { wr(fp, &v, 8); }
static void wd(FILE *fp, double v) { wr(fp, &v, 8); }
static void wv(FILE *fp, const std::vector<double> &v) {
    wi(fp, (long long)v.size());
    wr(fp, v.data(), v.size() * 8);
}

static void dump_state(SolverManager &SM, Settings &S, const std::string &path, double dt, long long step) {
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) {
        perror(path.c_str());
        exit(2);
    }
    auto &em = *VX_GET(SM, SM_em);
    wr(fp, "VXST0001", 8);
    wi(fp, step);
    wd(fp, S.time);
    wd(fp, dt);
    wd(fp, VX_GET(em, EM_ex0));
    int n = VX_GET(em, EM_xsize);
    wi(fp, n);
    wi(fp, VX_GET(em, EM_pre));
    wi(fp, VX_GET(em, EM_post));
    wv(fp, VX_GET(em, EM_By));
    wv(fp, VX_GET(em, EM_Bz));
    wv(fp, VX_GET(em, EM_Ey));
    wv(fp, VX_GET(em, EM_Ez));
    wv(fp, VX_GET(em, EM_Ay));
    wv(fp, VX_GET(em, EM_Az));
    wv(fp, VX_GET(em, EM_asq));
    std::vector<double> phi(VX_GET(em, EM_phi), VX_GET(em, EM_phi) + n);
    wv(fp, phi);
    wv(fp, VX_GET(em, EM_charge));
    wv(fp, VX_GET(em, EM_J));
    wv(fp, VX_GET(em, EM_neut));
    auto &meshes = VX_GET(SM, SM_meshes);
    wi(fp, (long long)meshes.size());
    for (auto &mesh : meshes) {
        wi(fp, (long long)mesh->levels.size());
        for (auto &lvl : mesh->levels) {
            wi(fp, (long long)lvl->rectangles.size());
            for (auto &rp : lvl->rectangles) {
                Rectangle &R = *rp;
                wi(fp, R.x_pos);
                wi(fp, R.p_pos);
                wi(fp, R.n_x);
                wi(fp, R.n_p);
                wi(fp, VX_GET(R, R_depth));
                wi(fp, VX_GET(R, R_up));
                wi(fp, VX_GET(R, R_down));
                wi(fp, VX_GET(R, R_left));
                wi(fp, VX_GET(R, R_right));
                wv(fp, R.f);
            }
        }
    }
    fclose(fp);
}

// ---------------------------------------------------------------- driver
static std::map<std::string, std::string> parse_args(int argc, char **argv) {
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto eq = a.find('=');
        if (eq == std::string::npos) {
            fprintf(stderr, "bad argument %s (expected key=value)\n", a.c_str());
            exit(2);
        }
        kv[a.substr(0, eq)] = a.substr(eq + 1);
    }
    return kv;
}

int main(int argc, char **argv) {
    auto kv = parse_args(argc, argv);
    auto getd = [&](const char *k, double d) { return kv.count(k) ? std::stod(kv[k]) : d; };
    auto geti = [&](const char *k, long long d) { return kv.count(k) ? std::stoll(kv[k]) : d; };
#ifndef VX_HOOKS_PROBLEM
    P.L = getd("L", P.L);
    P.nx = (unsigned)geti("nx", P.nx);
    P.np = (unsigned)geti("np", P.np);
    P.Lfinest = (unsigned)geti("levels", P.Lfinest);
    P.r = (unsigned)geti("r", P.r);
    P.pmax = getd("pmax", P.pmax);
    P.dens = getd("dens", P.dens);
    P.x1 = getd("x1", P.x1);
    P.x2 = getd("x2", P.x2);
    P.x3 = getd("x3", P.x3);
    P.x4 = getd("x4", P.x4);
    P.Te = getd("Te", P.Te);
    P.p0 = getd("p0", P.p0);
    P.bdens = getd("bdens", P.bdens);
    P.bp0 = getd("bp0", P.bp0);
    P.bTe = getd("bTe", P.bTe);
    P.pert_amp = getd("pert_amp", P.pert_amp);
    P.pert_k = getd("pert_k", P.pert_k);
    P.a0 = getd("a0", P.a0);
    P.fwhm = getd("fwhm", P.fwhm);
    P.delay = getd("delay", P.delay);
    P.cfl = getd("cfl", P.cfl);
    P.minEff = getd("minEff", P.minEff);
    P.crit = getd("crit", P.crit);
    P.sizeWeight = getd("sizeWeight", P.sizeWeight);
    P.quadDepth = (int)geti("quadDepth", P.quadDepth);
    P.mi = getd("mi", P.mi);
    P.iTe = getd("iTe", P.iTe);
    P.ipmax = getd("ipmax", P.ipmax);
#else
    sin2_defaults(&HP);
    HP.nx = (uint32_t)geti("nx", HP.nx);
    HP.np = (uint32_t)geti("np", HP.np);
    HP.Lfinest = (uint32_t)geti("levels", HP.Lfinest);
    HP.L = getd("L", HP.L);
    HP.pad = getd("pad", HP.pad);
    HP.a0 = getd("a0", HP.a0);
    HP.ramp = getd("ramp", HP.ramp);
    HP.crit = getd("crit", HP.crit);
    HP.minEff = getd("minEff", HP.minEff);
#endif
    long long steps = geti("steps", 0);
    long long dump_every = geti("dump_every", 0);
    long long regrid_every = geti("regrid_every", 0);
    long long time_steps = geti("time_steps", 0);
    // diag_every=K: SolverManager::fileOutput and OutputRectangles at t = 0 and after every
    // K-th step, into output/ and output/rectangleData/ of the working directory.
    long long diag_every = geti("diag_every", 0);
#ifndef VX_HOOKS_PROBLEM
    P.diag = diag_every > 0;
#endif
    std::string dumpdir = kv.count("dumpdir") ? kv["dumpdir"] : "";

    Input grid;
    Particles particles;
    Output output;
    initialConditions(grid, particles, output);
    std::streambuf *old = std::cout.rdbuf();
    std::ostringstream sink;
    std::cout.rdbuf(sink.rdbuf());  // silence the banner and level table
    Settings settings(grid, particles, output);
#ifdef VX_HOOKS_PROBLEM
    settings_to_c(settings, VIEW);  // the Settings are complete (sizes, fMax)
#endif
    auto t_init0 = std::chrono::steady_clock::now();
    SolverManager SM(settings);
    auto t_init1 = std::chrono::steady_clock::now();
    std::cout.rdbuf(old);

    char name[512];
    if (!dumpdir.empty()) {
        snprintf(name, sizeof name, "%s/state_%05lld.bin", dumpdir.c_str(), 0LL);
        dump_state(SM, settings, name, 0.0, 0);
    }
    auto diag = [&] {
        SM.fileOutput(settings.time);
        SM.OutputRectangles(settings.time);
    };
    if (diag_every > 0) diag();
    for (long long s = 1; s <= steps; s++) {
        double dt = SM.CalculateDt(settings.cfl);
        SM.Advance(dt);
        bool regrid = regrid_every > 0 && (s % regrid_every) == 0;
        if (!dumpdir.empty() && dump_every > 0 && (s % dump_every == 0 || regrid)) {
            snprintf(name, sizeof name, "%s/state_%05lld.bin", dumpdir.c_str(), s);
            dump_state(SM, settings, name, dt, s);
        }
        if (diag_every > 0 && s % diag_every == 0) diag();
        if (regrid) {
            std::cout.rdbuf(sink.rdbuf());
            SM.reGrid(settings.time);
            std::cout.rdbuf(old);
            if (!dumpdir.empty()) {
                snprintf(name, sizeof name, "%s/regrid_%05lld.bin", dumpdir.c_str(), s);
                dump_state(SM, settings, name, dt, s);
            }
        }
    }
    if (time_steps > 0) {
        // Time SolverManager::Advance only: one warm-up step, then time_steps timed steps.
        double dt = SM.CalculateDt(settings.cfl);
        SM.Advance(dt);
        long long cells = 0;
        for (auto &mesh : VX_GET(SM, SM_meshes))
            for (auto &lvl : mesh->levels)
                for (auto &rp : lvl->rectangles) cells += (long long)rp->n_x * rp->n_p;
        std::vector<double> per;
        for (long long s = 0; s < time_steps; s++) {
            dt = SM.CalculateDt(settings.cfl);
            auto a = std::chrono::steady_clock::now();
            SM.Advance(dt);
            auto b = std::chrono::steady_clock::now();
            per.push_back(std::chrono::duration<double>(b - a).count());
        }
        std::sort(per.begin(), per.end());
        printf("{\"cells\": %lld, \"steps\": %lld, \"best_s\": %.6f, \"median_s\": %.6f, \"threads\": %d, \"init_s\": %.3f}\n",
               cells, time_steps, per.front(), per[per.size() / 2], omp_get_max_threads(),
               std::chrono::duration<double>(t_init1 - t_init0).count());
    }
    return 0;
}
