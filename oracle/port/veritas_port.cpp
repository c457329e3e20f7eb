// ORACLE / TEST INFRASTRUCTURE — CPU restatement of the Veritas Vlasov–Maxwell step.
//
// Not part of the product: tests compare the CUDA path against it, and bench.py times
// it on the host cores as the CPU baseline ("kind": "port").  It restates, in plain
// C++/OpenMP, the per-step algorithm of the reference for one species on its
// block-structured AMR hierarchy, and the construction of that hierarchy at t = 0:
//   SolverManager::SolverManager      SolverManager.cpp:8-26
//   Mesh::Mesh, updateHierarchy(true)  Mesh.cpp:8-50, 132-210 (flagging, clustering by
//                                      Mesh.cpp:298-792, promoteHierarchyToMesh :794-875)
//   Rectangle::getError / weights      Rectangle.cpp:866-890, 68-74; Rectangle.hpp:128-130
//   Settings::DetermineMaximum         Settings.cpp:181-194
//   Mesh::PushData / PushBoundaryC     Mesh.cpp:91-106, 904-917 (ghost fills, coarse-fine
//                                      fluxes, limiter exchange; Rectangle.cpp:307-614,
//                                      1032-1253, 1625-1960)
//   SolverManager::Advance            SolverManager.cpp:28-39
//   EMFieldSolver::AssembleRhoAndJ     EMSolver.cpp:104-122
//   Rectangle::CalculateRhoAndJ (MKL)  Rectangle.cpp:157-237, 276-281
//   EMFieldSolver::UpdatePotential     EMSolver.cpp:156-192  (LU: oracle/lu_exact.hpp)
//   Rectangle::FCTTimeStep             Rectangle.cpp:1255-1623
//   EMFieldSolver::RGKStep             EMSolver.cpp:194-619
//   EMFieldSolver::EstimateCFLBound    EMSolver.cpp:631-664
//   Rectangle::InitializeDistribution  Rectangle.cpp:616-665
//   Settings::UpdateTime               Settings.cpp:166-179
// Each floating-point expression keeps the reference's operations and order, so with
// -ffp-contract=off the results are bit-identical to the reference build (which links
// the same LU restatement through its MKL header shim).  Pinned against the reference's
// own dumps by tests/test_oracle_port.py.
//
// Command line: the parity harness's key=value problem arguments, plus
//   load=<state file>  start from a VXST0001 state instead of t=0
//   dts=a,b,c          use these step sizes instead of the CFL bound
//   steps=N dump_every=K dumpdir=D time_steps=M warmup=W
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iterator>
#include <limits>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../lu_exact.hpp"

namespace {

// Constants as the reference defines them (veritas.hpp:22-30).
const double eps0_inv = 1.1294e+11;
const double eps0 = 8.854187817e-12;
const double mu_inv = 795774.715482;
const double cs = 299792458.0;
const double c_inv = 3.33564095e-9;
const double DPI = 6.28318530718;

const double kMe = 9.10938291e-31;
const double kQe = -1.60217657e-19;
const double kKeV = 1.602176565e-16;

struct Params {
    double lambda = 1e-6, L = 100.0;
    unsigned nx = 2048, np = 256, Lfinest = 1, r = 2;
    double pmax = 2.0, dens = 0.01, x1 = 15, x2 = 20, x3 = 80, x4 = 85, Te = 1.0, p0 = 0.0;
    double pert_amp = 0.0, pert_k = 1.0, a0 = 1.0, fwhm = 10.0, delay = 10.0;
    double cfl = 0.5, minEff = 0.75, crit = 1e-6, sizeWeight = 1.0;
    int quadDepth = 2;
    double bdens = 0.0, bp0 = 0.0, bTe = 1.0;
};

// ------------------------------------------------------------------ problem hooks
struct Problem {
    Params P;
    double m, q, dp, pmin, dx, n0, sigma, pdrift, A0, bsigma, bdrift;
    int maxDepth, quadDepth;
    unsigned x_size, p_size, r;

    void setup() {
        m = kMe;
        q = kQe;
        x_size = P.nx;
        p_size = P.np;
        r = P.r;
        maxDepth = (int)P.Lfinest - 1;
        double mc = m * cs;
        dp = 2.0 * P.pmax * mc / p_size;
        pmin = -P.pmax * mc;
        dx = P.L * P.lambda / x_size;
        quadDepth = P.quadDepth;
        double T = P.lambda / cs;
        double omega = DPI / T;
        double Nc = omega * omega * m * eps0 / (q * q);
        n0 = P.dens * Nc;
        sigma = m * (P.Te * kKeV);
        pdrift = P.p0 * mc;
        A0 = P.a0 * mc / std::fabs(q);
        bsigma = m * (P.bTe * kKeV);
        bdrift = P.bp0 * mc;
    }
    double slab(double xl) const {
        double s;
        if (xl <= P.x1 || xl >= P.x4) s = 0.0;
        else if (xl < P.x2) s = (xl - P.x1) / (P.x2 - P.x1);
        else if (xl <= P.x3) s = 1.0;
        else s = (P.x4 - xl) / (P.x4 - P.x3);
        if (P.pert_amp != 0.0) s = s * (1.0 + P.pert_amp * std::sin(DPI * P.pert_k * xl / P.L));
        return s;
    }
    double init_f(double x, double p) const {
        double ne = n0 * slab(x / P.lambda);
        double d = p - pdrift;
        double v = ne * std::exp(-(d * d) / (2.0 * sigma)) / std::sqrt(DPI * sigma);
        if (P.bdens != 0.0) {
            double db = p - bdrift;
            v += P.bdens * ne * std::exp(-(db * db) / (2.0 * bsigma)) / std::sqrt(DPI * bsigma);
        }
        return v;
    }
    double BY(double, double) const { return 0.0; }
    double BZ(double x, double t) const {
        double T = P.lambda / cs;
        double k = DPI / P.lambda;
        double omega = cs * k;
        double F = P.fwhm * T;
        double tau = (t - x / cs) - P.delay * T;
        double c4 = 4.0 * std::log(2.0) / (F * F);
        double g = std::exp(-c4 * tau * tau);
        double gp = -2.0 * c4 * tau * g;
        double ph = omega * t - k * x;
        return A0 * (k * g * std::sin(ph) - (gp / cs) * std::cos(ph));
    }
    double GetDx(int level) const { return std::pow(r, level - maxDepth) * dx; }
    double GetDp(int level) const { return std::pow(r, level - maxDepth) * dp; }
    int GetXSize(int level) const { return x_size * std::pow(r, -level + maxDepth); }
    int GetPSize(int level) const { return p_size * std::pow(r, -level + maxDepth); }
};

// ------------------------------------------------------------------ patch
// One patch: SoA planes of (nx+4) x (np+4) doubles, p fastest.
struct Patch {
    int nx, np, x_pos = 0, p_pos = 0, depth, rtb, r = 2, species = 0;
    bool up = true, down = true, left = true, right = true;
    int W;  // row width np + 4
    std::vector<double> f[3], gam, ex, fx, ep, fp, FxH[6], FpH[6], FxL, FpL, FxDS, FpDS, Rp, Rm, Cx, Cp;
    std::vector<double> chargeR, currentR, relc, refc;
    double dx, dp, dx_inv, dp_inv, pmin, q, m, cc, g2;
    // AMR connectivity (Rectangle.hpp:8-12): neighbour patch index per edge entry (-1:
    // the domain boundary), "same level" flags, finer patch per cell / face, masks
    std::vector<int> xm, xp, pm, pp;
    std::vector<char> sxm, sxp, spm, spp;
    std::vector<int> finer, finer_x, finer_p;
    std::vector<char> nested, ifx, ifp;
    size_t id(int i, int j) const { return (size_t)(i + 2) * W + (j + 2); }
    void alloc() {
        W = np + 4;
        size_t N = (size_t)(nx + 4) * W;
        xm.assign(np / r + 2, -1);
        xp.assign(np / r + 2, -1);
        pm.assign(nx / r, -1);
        pp.assign(nx / r, -1);
        sxm.assign(np / r + 2, 1);
        sxp.assign(np / r + 2, 1);
        spm.assign(nx / r, 1);
        spp.assign(nx / r, 1);
        finer.assign(N, -1);
        finer_x.assign(N, -1);
        finer_p.assign(N, -1);
        nested.assign(N, 0);
        ifx.assign(N, 0);
        ifp.assign(N, 0);
        for (auto &v : f) v.assign(N, 0.0);
        for (auto *v : {&gam, &ex, &fx, &ep, &fp, &FxL, &FpL, &FxDS, &FpDS, &Rp, &Rm, &Cx, &Cp}) v->assign(N, 0.0);
        for (int s = 0; s < 6; s++) {
            FxH[s].assign(N, 0.0);
            FpH[s].assign(N, 0.0);
        }
        chargeR.assign((size_t)nx * rtb, 0.0);
        currentR.assign((size_t)nx * rtb, 0.0);
    }
};

struct Fields {
    int n, pre, post, nf;
    std::vector<double> By, Bz, Ey, Ez, Ay, Az, asq, phi, charge, J, neut;
    double Ex0 = 0.0, fcoef;
    size_t I(int i, int slot) const { return (size_t)slot * nf + i; }
};

// ------------------------------------------------------------------ numerics
inline double vmax(double a, double b) { return (a > b) ? a : b; }
inline double vmin(double a, double b) { return (a < b) ? a : b; }

double weno(double f1, double f2, double f3, double f4, bool right) {
    double fL = (1.0 / 6) * (-f1 + 5 * f2 + 2 * f3);
    double fR = (1.0 / 6) * (2 * f2 + 5 * f3 - f4);
    double AL = f1 - 2 * f2 + f3;
    double BL = f3 - f1;
    double AR = f2 - 2 * f3 + f4;
    double BR = f4 - f2;
    double bL = 4.0 / 3 * (AL * AL) + 0.5 * AL * BL + 0.25 * (BL * BL);
    double bR = 4.0 / 3 * (AR * AR) - 0.5 * AR * BR + 0.25 * (BR * BR);
    double mm = 1.0e-10;
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
    double wL0 = wL * (0.75 + wL * (wL - 0.5));
    double wR0 = wR * (0.75 + wR * (wR - 0.5));
    double pick = right ? ((wL0 > wR0) ? wL0 : wR0) : ((wL0 < wR0) ? wL0 : wR0);
    double fwl = pick / (wL0 + wR0);
    double fwr = 1 - fwl;
    return fwl * fL + fwr * fR;
}

// Rectangle::GetWenoEdgeValue (Rectangle.cpp:943-977), used by the fluxes a coarse
// patch takes from a finer one.
double weno_max(double f1, double f2, double f3, double f4, bool right) {
    double fL = (1.0 / 6) * (-f1 + 5 * f2 + 2 * f3);
    double fR = (1.0 / 6) * (2 * f2 + 5 * f3 - f4);
    double AL = f1 - 2 * f2 + f3;
    double BL = f3 - f1;
    double AR = f2 - 2 * f3 + f4;
    double BR = f4 - f2;
    double bL = 4.0 / 3 * (AL * AL) + 0.5 * AL * BL + 0.25 * (BL * BL);
    double bR = 4.0 / 3 * (AR * AR) - 0.5 * AR * BR + 0.25 * (BR * BR);
    double mm(1.0e-10);
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
    double wL0 = wL * (0.75 + wL * (wL - 0.5));
    double wR0 = wR * (0.75 + wR * (wR - 0.5));
    if (right) {
        wL = std::max(wL0, wR0) / (wL0 + wR0);
        wR = 1 - wL;
    } else {
        wL = std::min(wL0, wR0) / (wL0 + wR0);
        wR = 1 - wL;
    }
    return (wL * (fL) + wR * (fR));
}

double face_a(double f1, double f2, double f3, double f4) {
    double fL = (1.0 / 6) * (-f1 + 5 * f2 + 2 * f3);
    double fR = (1.0 / 6) * (2 * f2 + 5 * f3 - f4);
    double AL = f1 - 2 * f2 + f3;
    double BL = f3 - f1;
    double AR = f2 - 2 * f3 + f4;
    double BR = f4 - f2;
    double bL = 4.0 / 3 * (AL * AL) + 0.5 * AL * BL + 0.25 * (BL * BL);
    double bR = 4.0 / 3 * (AR * AR) - 0.5 * AR * BR + 0.25 * (BR * BR);
    double mm(1.0e-10);
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
    return wL * fL + wR * fR;
}

struct Solver {
    Problem pr;
    std::vector<Patch> patches;        // every patch of the (single) species
    std::vector<std::vector<int>> lv;  // lv[depth]: patch indices in the reference's level order
    Fields F;
    vxo::SparseLU lu;
    double time = 0.0;

    double asq_face(int x) const { return F.asq[std::min(std::max(x, 0), F.n)]; }
    double efield(int i) const {
        const int n = F.n;
        int ip1 = i + 1, im1 = i - 1, ip2 = i + 2, im2 = i - 2;
        ip1 = (ip1 > -1) ? ip1 : (ip1 + n);
        im1 = (im1 > -1) ? im1 : (im1 + n);
        ip2 = (ip2 > -1) ? ip2 : (ip2 + n);
        im2 = (im2 > -1) ? im2 : (im2 + n);
        ip1 = (ip1 < n) ? ip1 : (ip1 - n);
        im1 = (im1 < n) ? im1 : (im1 - n);
        ip2 = (ip2 < n) ? ip2 : (ip2 - n);
        im2 = (im2 < n) ? im2 : (im2 - n);
        const double *P = F.phi.data();
        return -F.fcoef * (8 * (P[ip1] - P[im1]) - P[ip2] + P[im2]) + F.Ex0;
    }
    double patch_efield(const Patch &P, int i) const {
        int x = P.rtb * (i + P.x_pos);
        double t = 0.0;
        for (int k = 0; k < P.rtb; k++) t += efield(x + k);
        return t * (1.0 / P.rtb);
    }
    double cell_asq(int x) const {
        int i = x + F.pre;
        i = i > -1 ? i : 0;
        i = i < F.nf ? i : F.nf - 1;
        double ay = F.Ay[F.I(i, 1)], az = F.Az[F.I(i, 1)];
        return (ay * ay) + (az * az);
    }

    Patch make_patch(int depth, int x_pos, int p_pos, int nx, int np) {
        Patch P;
        P.nx = nx;
        P.np = np;
        P.x_pos = x_pos;
        P.p_pos = p_pos;
        P.depth = depth;
        P.r = (int)pr.r;
        P.rtb = (int)std::pow(pr.r, depth);
        P.dx = pr.GetDx(depth);
        P.dp = pr.GetDp(depth);
        P.dx_inv = 1 / P.dx;
        P.dp_inv = 1 / P.dp;
        P.pmin = pr.pmin;
        P.q = pr.q;
        P.m = pr.m;
        P.cc = cs * cs * pr.m;
        double m_inv = 1 / pr.m;
        P.g2 = (m_inv * c_inv) * (m_inv * c_inv);
        P.relc.assign(3 * P.rtb, 0.0);
        for (int i = 0; i < P.rtb; i++) {  // Rectangle.cpp:103-110
            double rb = P.rtb;
            double tl = -0.5 + i / rb;
            double tr = -0.5 + (i + 1.0) / rb;
            P.relc[3 * i] = (tl + tr) * 0.5;
            P.relc[3 * i + 1] = (tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12);
            P.relc[3 * i + 2] = (tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25;
        }
        P.refc.assign(3 * P.r, 0.0);
        for (int i = 0; i < P.r; i++) {  // Rectangle.cpp:94-101
            double tl = -0.5 + i / (double)P.r;
            double tr = -0.5 + (i + 1.0) / (double)P.r;
            P.refc[3 * i] = (tl + tr) * 0.5;
            P.refc[3 * i + 1] = (tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12);
            P.refc[3 * i + 2] = (tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25;
        }
        P.alloc();
        return P;
    }

    void setup() {
        pr.setup();
        const int base = pr.maxDepth;
        patches.push_back(make_patch(base, 0, 0, pr.GetXSize(base), pr.GetPSize(base)));
        lv.assign(pr.maxDepth + 1, {});
        lv[base].push_back(0);
        F.n = pr.x_size * std::pow(pr.r, pr.maxDepth);
        F.pre = std::max(std::floor(0.0 / pr.GetDx(0)), 2.0);
        F.post = std::max(std::floor(0.0 / pr.GetDx(0)), 2.0);
        F.nf = F.n + F.pre + F.post;
        for (auto *v : {&F.By, &F.Bz, &F.Ey, &F.Ez, &F.Ay, &F.Az}) v->assign((size_t)F.nf * 8, 0.0);
        F.asq.assign(F.n + 1, 0.0);
        for (auto *v : {&F.phi, &F.charge, &F.J, &F.neut}) v->assign(F.n, 0.0);
        F.fcoef = 1.0 / (12 * pr.GetDx(0));
        const int n = F.n;
        const double w1 = -16.0 / 30.0 / 0.4, w2 = 1.0 / 30.0 / 0.4, w3 = 1 / 0.4;
        std::vector<std::vector<std::pair<int, double>>> rows(n);
        std::vector<std::map<int, double>> acc(n);
        auto put = [&](int col, int row, double v) { acc[row][col] = v; };
        for (int i = 2; i < n - 2; i++) {
            put(i, i, w3);
            put(i, i + 1, w1);
            put(i, i - 1, w1);
            put(i, i + 2, w2);
            put(i, i - 2, w2);
        }
        put(0, 0, 1.0);
        put(1, 1, w3), put(1, 2, w1), put(1, 0, w1), put(1, 3, w2), put(1, n - 1, w2);
        put(n - 2, n - 2, w3), put(n - 2, n - 1, w1), put(n - 2, n - 3, w1), put(n - 2, 0, w2), put(n - 2, n - 4, w2);
        put(n - 1, n - 1, w3), put(n - 1, 0, w1), put(n - 1, n - 2, w1), put(n - 1, 1, w2), put(n - 1, n - 3, w2);
        for (int rr = 0; rr < n; rr++)
            for (auto &kv : acc[rr]) rows[rr].push_back({kv.first, kv.second});
        lu.factor_rows(rows);
    }

    // SolverManager::SolverManager (SolverManager.cpp:8-26): the hierarchy (Mesh::Mesh),
    // the ghost fill, then EMFieldSolver::EnforceChargeNeutralization (EMSolver.cpp:621-629).
    void init_distribution() {
        build_hierarchy();
        push_data(1);
        assemble();
        for (int i = 0; i < F.n; i++) F.neut[i] = -F.charge[i];
        std::fill(F.J.begin(), F.J.end(), 0.0);
    }

    // ---------------------------------------------------------------- AMR connectivity
    static bool on_line(int x, int y1, int y2) { return ((x - y1) > -1) && ((y2 - x) > -1); }

    // Rectangle::CalculateConnectivityFromFiner (Rectangle.cpp:768-864): `c` is a patch,
    // `fi` a patch one level finer.
    void connect_finer(int ci, int fi) {
        Patch &C = patches[ci], &Fp = patches[fi];
        const int r = C.r;
        const int x2 = Fp.x_pos / r - C.x_pos, p2 = Fp.p_pos / r - C.p_pos;
        const int nx2 = Fp.nx / r, np2 = Fp.np / r;
        const int lower_x = std::max(0, x2), upper_x = std::min(C.nx, x2 + nx2);
        const int lower_p = std::max(0, p2), upper_p = std::min(C.np, p2 + np2);
        for (int i = lower_x; i < upper_x; i++)
            for (int j = lower_p; j < upper_p; j++) {
                C.nested[C.id(i, j)] = 1;
                C.finer[C.id(i, j)] = fi;
            }
        const int last = (int)Fp.xp.size() - 1;
        if ((x2 + nx2) < (C.nx + 1) && (x2 + nx2) > -1)
            for (int i = lower_p; i < upper_p; i++) {
                C.finer_x[C.id(x2 + nx2, i)] = fi;
                C.ifx[C.id(x2 + nx2, i)] = 1;
            }
        if ((x2 + nx2) < C.nx && (x2 + nx2) > -1) {
            for (int i = lower_p; i < upper_p; i++) Fp.xp[i - p2 + 1] = ci, Fp.sxp[i - p2 + 1] = 0;
            if (on_line(p2 - 1, 0, C.np - 1)) Fp.xp[0] = ci, Fp.sxp[0] = 0;
            if (on_line(p2 + np2, 0, C.np - 1)) Fp.xp[last] = ci, Fp.sxp[last] = 0;
        }
        if (x2 < (C.nx + 1) && x2 > -1)
            for (int i = lower_p; i < upper_p; i++) {
                C.finer_x[C.id(x2, i)] = fi;
                C.ifx[C.id(x2, i)] = 1;
            }
        if (x2 < (C.nx + 1) && x2 > 0) {
            for (int i = lower_p; i < upper_p; i++) Fp.xm[i - p2 + 1] = ci, Fp.sxm[i - p2 + 1] = 0;
            if (on_line(p2 - 1, 0, C.np - 1)) Fp.xm[0] = ci, Fp.sxm[0] = 0;
            if (on_line(p2 + np2, 0, C.np - 1)) Fp.xm[last] = ci, Fp.sxm[last] = 0;
        }
        if ((p2 + np2) < (C.np + 1) && (p2 + np2) > -1)
            for (int i = lower_x; i < upper_x; i++) {
                C.finer_p[C.id(i, p2 + np2)] = fi;
                C.ifp[C.id(i, p2 + np2)] = 1;
            }
        if ((p2 + np2) < C.np && (p2 + np2) > -1)
            for (int i = lower_x; i < upper_x; i++) Fp.pp[i - x2] = ci, Fp.spp[i - x2] = 0;
        if (p2 < (C.np + 1) && p2 > -1)
            for (int i = lower_x; i < upper_x; i++) {
                C.finer_p[C.id(i, p2)] = fi;
                C.ifp[C.id(i, p2)] = 1;
            }
        if (p2 < (C.np + 1) && p2 > 0)
            for (int i = lower_x; i < upper_x; i++) Fp.pm[i - x2] = ci, Fp.spm[i - x2] = 0;
    }

    // Rectangle::CalculateConnectivitySame (Rectangle.cpp:671-766)
    void connect_same(int ai, int bi) {
        Patch &A = patches[ai];
        const Patch &B = patches[bi];
        const int r = A.r;
        const int xr = B.x_pos - A.x_pos, pr_ = B.p_pos - A.p_pos;
        const int lx = (int)A.xm.size() - 1;
        if (xr == A.nx) {
            int lower = std::max(B.p_pos, A.p_pos), upper = std::min(A.p_pos + A.np, B.p_pos + B.np);
            if (on_line(-1, pr_, pr_ + B.np - 1)) A.xp[0] = bi, A.sxp[0] = 1;
            if (on_line(A.np, pr_, pr_ + B.np - 1)) A.xp[lx] = bi, A.sxp[lx] = 1;
            for (; lower < upper; lower += r) A.xp.at((lower - A.p_pos) / r + 1) = bi, A.sxp.at((lower - A.p_pos) / r + 1) = 1;
        }
        if (xr == -B.nx) {
            int lower = std::max(B.p_pos, A.p_pos), upper = std::min(A.p_pos + A.np, B.p_pos + B.np);
            if (on_line(-1, pr_, pr_ + B.np - 1)) A.xm[0] = bi, A.sxm[0] = 1;
            if (on_line(A.np, pr_, pr_ + B.np - 1)) A.xm[lx] = bi, A.sxm[lx] = 1;
            for (; lower < upper; lower += r) A.xm.at((lower - A.p_pos) / r + 1) = bi, A.sxm.at((lower - A.p_pos) / r + 1) = 1;
        }
        if (pr_ == A.np) {
            int lower = std::max(B.x_pos, A.x_pos), upper = std::min(A.x_pos + A.nx, B.x_pos + B.nx);
            if (on_line(-1, xr, xr + B.nx - 1)) A.xm[lx] = bi, A.sxm[lx] = 1;
            if (on_line(A.nx, xr, xr + B.nx - 1)) A.xp[lx] = bi, A.sxp[lx] = 1;
            for (; lower < upper; lower += r) A.pp.at((lower - A.x_pos) / r) = bi, A.spp.at((lower - A.x_pos) / r) = 1;
        }
        if (pr_ == -B.np) {
            int lower = std::max(B.x_pos, A.x_pos), upper = std::min(A.x_pos + A.nx, B.x_pos + B.nx);
            if (on_line(-1, xr, xr + B.nx - 1)) A.xm[0] = bi, A.sxm[0] = 1;
            if (on_line(A.nx, xr, xr + B.nx - 1)) A.xp[0] = bi, A.sxp[0] = 1;
            for (; lower < upper; lower += r) A.pm.at((lower - A.x_pos) / r) = bi, A.spm.at((lower - A.x_pos) / r) = 1;
        }
    }

    // Mesh::promoteHierarchyToMesh connectivity loops (Mesh.cpp:836-859) on patches whose
    // connectivity is still the constructor's (every edge on the domain boundary).
    void connect_keep_f() {
        for (int l = 0; l <= pr.maxDepth; l++)
            for (int rl : lv[l])
                if (l > 0)
                    for (int rf : lv[l - 1]) connect_finer(rl, rf);
        for (int l = 0; l <= pr.maxDepth; l++)
            for (int rl : lv[l])
                for (int rr : lv[l])
                    if (rl != rr) connect_same(rl, rr);
    }

    // ---------------------------------------------------------------- initial hierarchy
    // Mesh::Mesh (Mesh.cpp:8-50) in the reference's default configuration (MKLINIT 0):
    // the initial getError(init) keeps its flags in a private list (Mesh.cpp:272-287),
    // so the hierarchy starts as the base patch alone and gains its finer levels from
    // maxDepth rounds of flagging on quadrature-initialised data, every round
    // re-initialising every patch from the quadrature (promoteHierarchyToMesh(true)).
    typedef std::pair<int, int> Cell;  // (i, j) in a level's global coordinates
    struct Box {                       // Mesh's rect: lower-left and upper-right corners
        int x0, p0, x1, p1;
    };
    std::vector<std::vector<Box>> H;  // H[0] = the base level, coarse to fine
    double fmax = 0.0;

    // Settings::DetermineMaximum (Settings.cpp:181-194): the peak of f on the finest x grid at p = 0.
    void determine_maximum() {
        const double dx0 = pr.GetDx(0);
        double mv(0.0);
        for (int i = 0; i < pr.GetXSize(0); i++) {
            double t(pr.init_f((i + 0.5) * dx0, 0));
            mv = t > mv ? t : mv;
        }
        fmax = mv;
    }

    // Rectangle::InitializeDistribution (Rectangle.cpp:616-665, non-MKL loop)
    void quadrature(Patch &P) {
        const int nvals = std::pow(pr.r, P.depth + pr.quadDepth);
#pragma omp parallel for schedule(guided)
        for (int i = 0; i < P.nx; i++)
            for (int j = 0; j < P.np; j++) {
                double temp = 0.0;
                for (int k = 0; k < nvals; k++)
                    for (int l = 0; l < nvals; l++) {
                        double xp = ((0.5 + k) / nvals + i + P.x_pos) * P.dx;
                        double pp = P.pmin + P.dp * ((0.5 + l) / nvals + j + P.p_pos);
                        temp += pr.init_f(xp, pp);
                    }
                P.f[0][P.id(i, j)] = temp * (1 / std::pow(nvals, 2.0));
                P.f[1][P.id(i, j)] = temp * (1 / std::pow(nvals, 2.0));
            }
    }

    // Rectangle::getError (Rectangle.cpp:866-890) with ErrorEstimate (Rectangle.hpp:128-130)
    // and the weights of the Rectangle constructor (Rectangle.cpp:68-74).  The problem's
    // RefinementOverride is false.
    void patch_flags(const Patch &P, std::vector<Cell> &out) const {
        const double rr = pr.r;
        double w[5];
        w[0] = 0.5 / fmax * std::pow(rr, -0.5 * P.depth);
        w[1] = 0.5 / fmax * std::pow(rr, -0.5 * P.depth);
        w[2] = 0.5 / fmax * std::pow(rr, -2.0 * P.depth);
        w[3] = 0.5 / fmax * std::pow(rr, -2.0 * P.depth);
        w[4] = pr.P.sizeWeight / fmax * std::pow(rr, -pr.maxDepth + P.depth);
        int band = 0;
        for (int k = 0; k <= pr.maxDepth - P.depth; k++) band += std::pow(pr.r, k);
        band *= 3;
        const int ilo = std::max(P.x_pos, band), ihi = std::min(P.x_pos + P.nx, pr.GetXSize(P.depth) - band);
        const int jlo = std::max(P.p_pos, band), jhi = std::min(P.p_pos + P.np, pr.GetPSize(P.depth) - band);
        const double *f = P.f[1].data();
        for (int i = ilo; i < ihi; i++)
            for (int j = jlo; j < jhi; j++) {
                const int a = i - P.x_pos, b = j - P.p_pos;
                const double c = f[P.id(a, b)];
                double e = w[0] * std::fabs(f[P.id(a + 1, b)] - f[P.id(a - 1, b)]) +
                           w[1] * std::fabs(f[P.id(a, b + 1)] - f[P.id(a, b - 1)]) +
                           w[2] * std::fabs(f[P.id(a + 1, b)] - 2 * c + f[P.id(a - 1, b)]) +
                           w[3] * std::fabs(f[P.id(a, b + 1)] - 2 * c + f[P.id(a, b - 1)]) + w[4] * std::fabs(c);
                if (e > pr.P.crit) out.push_back(Cell(i, j));
            }
    }
    // Mesh::getError(lvl, false) (Mesh.cpp:289-294): hierarchy index -> depth maxDepth - lvl
    void level_flags(int lvl, std::vector<Cell> &out) const {
        for (int k : lv[pr.maxDepth - lvl]) patch_flags(patches[k], out);
    }

    // Mesh::interpRectanglesUp (Mesh.cpp:298-313): close the upper corner and scale the
    // boxes found on hierarchy index lvl to the grid of lvl + 1 (int *= double truncates).
    void boxes_up(std::vector<Box> &bs, int lvl) const {
        const int n0 = pr.GetXSize(pr.maxDepth - lvl), m0 = pr.GetPSize(pr.maxDepth - lvl);
        const int n1 = pr.GetXSize(pr.maxDepth - (lvl + 1)), m1 = pr.GetPSize(pr.maxDepth - (lvl + 1));
        for (Box &b : bs) {
            b.x1 += 1;
            b.p1 += 1;
            b.x0 *= (n1 / double(n0));
            b.p0 *= (m1 / double(m0));
            b.x1 *= (n1 / double(n0));
            b.p1 *= (m1 / double(m0));
        }
    }
    // Mesh::mergeDownFlaggedData (Mesh.cpp:315-339): the cells of hierarchy index lvl that
    // lie under a box of index lvl + 2 widened by two ratios (upper x bound one further).
    void merge_down(int lvl, const Box &b, std::vector<Cell> &out) const {
        const int n0 = pr.GetXSize(pr.maxDepth - lvl), m0 = pr.GetPSize(pr.maxDepth - lvl);
        const int n2 = pr.GetXSize(pr.maxDepth - (lvl + 2)), m2 = pr.GetPSize(pr.maxDepth - (lvl + 2));
        const int w = 2 * (int)pr.r;
        for (int i = b.x0 - w; i <= b.x1 + w + 1; i++)
            for (int j = b.p0 - w; j <= b.p1 + w; j++) {
                int ic = i * (n0 / double(n2));
                int jc = j * (m0 / double(m2));
                if (ic > -1 && ic < n0 && jc > -1 && jc < m0) out.push_back(Cell(ic, jc));
            }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }

    // Mesh::getExtrema (Mesh.cpp:626-642)
    static Box extrema(const std::vector<Cell> &c) {
        Box b{c[0].first, c[0].second, c[0].first, c[0].second};
        for (const Cell &x : c) {
            b.x0 = std::min(b.x0, x.first);
            b.x1 = std::max(b.x1, x.first);
            b.p0 = std::min(b.p0, x.second);
            b.p1 = std::max(b.p1, x.second);
        }
        return b;
    }
    // Mesh::hasHole (Mesh.cpp:597-624): the first zero run of a signature.  Returns found
    // and (start, finish): the entry before the run (or 0 at the edge) and the first entry
    // after it (or the last entry).
    static bool first_gap(const std::vector<int> &sig, int &start, int &finish) {
        start = finish = 0;
        size_t z = 0;
        while (z < sig.size() && sig[z] != 0) z++;
        if (z == sig.size()) return false;
        start = z == 0 ? 0 : (int)z - 1;
        size_t e = z;
        while (e < sig.size() && sig[e] == 0) e++;
        finish = e == sig.size() ? (int)e - 1 : (int)e;
        return true;
    }
    // The sign-change search of Mesh::identifyInflection (Mesh.cpp:449-595) along one
    // direction.  lap is the signature's discrete Laplacian.  Returns -1 when the
    // signature is too short to look at, 0 when it has no sign change (bisect), 1 with
    // (index, size) of the chosen change otherwise; `far` is the distance the reference
    // starts its closest-to-centre search from (INT_MAX along x, 32767 along p).
    static int best_inflection(const std::vector<int> &lap, int far, int &index, int &size) {
        index = size = 0;
        const int n = (int)lap.size();
        if (n <= 2) return -1;
        std::vector<int> at, mag;
        for (int i = 0; i + 1 < n; i++) {
            const int a = lap[i], b = lap[i + 1];
            const int sa = (a > 0) - (a < 0), sb = (b > 0) - (b < 0);
            if (a != 0 && b != 0 && sa != sb) {
                at.push_back(i);
                mag.push_back(std::abs(b - a));
            }
        }
        if (at.empty()) return 0;
        if (at.size() == 1) {
            index = at[0];
            size = mag[0];
            return 1;
        }
        const int top = *std::max_element(mag.begin(), mag.end());
        const int ties = (int)std::count(mag.begin(), mag.end(), top);
        int pick = 0;
        if (ties > 1) {
            int best = far;
            const int mid = n / 2;  // the reference's centre: the Laplacian's length / 2
            for (size_t k = 0; k < at.size(); k++)
                if (best > std::abs(at[k] - mid)) {
                    best = std::abs(at[k] - mid);
                    pick = (int)k;
                }
        } else {
            pick = (int)(std::max_element(mag.begin(), mag.end()) - mag.begin());
        }
        index = at[pick];
        size = mag[pick];
        return 1;
    }
    static std::vector<int> laplacian(const std::vector<int> &sig) {
        std::vector<int> d;
        if (sig.size() >= 3) {
            d.resize(sig.size() - 2);
            for (size_t h = 1; h + 1 < sig.size(); h++) d[h - 1] = sig[h - 1] + sig[h + 1] - 2 * sig[h];
        }
        return d;
    }
    static bool inside(const Cell &c, const Box &b) {
        return c.first >= b.x0 && c.first <= b.x1 && c.second >= b.p0 && c.second <= b.p1;
    }
    // Mesh::splitRectangle (Mesh.cpp:644-792): recursive cuts (holes first, the larger of
    // the two when both directions have one; then the largest signature inflection;
    // bisection of the long side last) until a box is efficient enough or too small.
    std::vector<Box> split(const Box &b, const std::vector<Cell> &cells) const {
        const double cellsIn = double((b.x1 - b.x0 + 1) * (b.p1 - b.p0 + 1));
        if (cells.size() / cellsIn > pr.P.minEff) return {b};
        std::vector<int> sx(b.x1 - b.x0 + 1, 0), sp(b.p1 - b.p0 + 1, 0);
        for (const Cell &c : cells) {
            sx.at(c.first - b.x0)++;
            sp.at(c.second - b.p0)++;
        }
        int hx0, hx1, hp0, hp1;
        const bool gx = first_gap(sx, hx0, hx1), gp = first_gap(sp, hp0, hp1);
        hx0 += b.x0, hx1 += b.x0, hp0 += b.p0, hp1 += b.p0;
        Box one, two;
        bool cutx;
        int cut_lo = 0, cut_hi = 0;  // one ends at cut_lo, two starts at cut_hi
        if (gx || gp) {
            cutx = gx && (!gp || std::abs(hx1 - hx0) > std::abs(hp1 - hp0));
            cut_lo = cutx ? hx0 : hp0;
            cut_hi = cutx ? hx1 : hp1;
        } else {
            // Mesh::computeSignatures builds the Laplacians only for boxes at least three
            // cells long in that direction (Mesh.cpp:412-441)
            const std::vector<int> lx = (b.x1 - b.x0 >= 2) ? laplacian(sx) : std::vector<int>();
            const std::vector<int> lp = (b.p1 - b.p0 >= 2) ? laplacian(sp) : std::vector<int>();
            int ix, mx, ip, mp;
            const int kx = best_inflection(lx, std::numeric_limits<int>::max(), ix, mx);
            const int kp = best_inflection(lp, 32767, ip, mp);
            if (kx == 0 && kp == 0) {  // bisect the long side
                const double lxd = b.x1 - b.x0, lpd = b.p1 - b.p0;
                cutx = lxd > lpd;
                const double at = cutx ? std::floor((lxd / 2) + b.x0) : std::floor((lpd / 2) + b.p0);
                cut_lo = (int)at;
                cut_hi = (int)at + 1;
            } else if ((lx.size() <= 2 && lp.size() <= 2) || (mx == 0 && mp == 0)) {
                return {b};
            } else {
                cutx = mx > mp;
                cut_lo = cutx ? ix + b.x0 + 1 : ip + b.p0 + 1;
                cut_hi = cut_lo + 1;
            }
        }
        if (cutx) {
            one = Box{b.x0, b.p0, cut_lo, b.p1};
            two = Box{cut_hi, b.p0, b.x1, b.p1};
        } else {
            one = Box{b.x0, b.p0, b.x1, cut_lo};
            two = Box{b.x0, cut_hi, b.x1, b.p1};
        }
        std::vector<Cell> c1, c2;
        for (const Cell &c : cells) (inside(c, one) ? c1 : c2).push_back(c);
        std::vector<Box> out;
        if (!c1.empty()) out = split(one, c1);
        if (!c2.empty()) {
            auto more = split(two, c2);
            out.insert(out.end(), more.begin(), more.end());
        }
        return out;
    }

    // Mesh::promoteHierarchyToMesh(true) (Mesh.cpp:794-875): patches for every box (depth 0
    // the finest; a hierarchy shorter than maxDepth + 1 levels leaves the finest depths
    // empty and compares its edges against the sizes of its own depth count), every patch
    // from the quadrature, connectivity, the ghost fill and f0 = f1 (FCTTimeStep(0,-1,3)).
    void promote() {
        const int N = (int)H.size() - 1, empty = pr.maxDepth - N;
        patches.clear();
        lv.assign(pr.maxDepth + 1, {});
        for (int l = N; l >= 0; l--) {
            const int depth = N - l + empty;
            const int xs = pr.GetXSize(N - l), ps = pr.GetPSize(N - l);
            for (const Box &b : H[l]) {
                Patch P = make_patch(depth, b.x0, b.p0, b.x1 - b.x0, b.p1 - b.p0);
                P.up = b.p1 == ps;
                P.down = b.p0 == 0;
                P.left = b.x0 == 0;
                P.right = b.x1 == xs;
                lv[depth].push_back((int)patches.size());
                patches.push_back(std::move(P));
            }
        }
        for (auto &P : patches) quadrature(P);
        connect_keep_f();
        push_data(1);
        for (auto &P : patches) P.f[0] = P.f[1];
    }

    // Mesh::updateHierarchy(true) (Mesh.cpp:132-210)
    void update_hierarchy() {
        const int top = (int)H.size() - 1;
        std::vector<Cell> cells;
        for (int l = top; l > -1; l--) {
            if (l < (int)H.size() - 2) {
                std::vector<Cell> own, under;
                if (H.size() > 2)
                    for (const Box &b : H.at(l + 2)) {
                        std::vector<Cell> t;
                        merge_down(l, b, t);
                        under.insert(under.end(), t.begin(), t.end());
                    }
                level_flags(l, own);
                std::sort(own.begin(), own.end());
                // `under` is a concatenation of sorted runs, not sorted itself; the
                // reference passes it to set_union as it is
                std::set_union(own.begin(), own.end(), under.begin(), under.end(), std::back_inserter(cells));
            } else {
                level_flags(l, cells);
            }
            if (!cells.empty()) {
                std::vector<Box> found = split(extrema(cells), cells);
                if (l == top) {
                    if (l < pr.maxDepth) {
                        boxes_up(found, l);
                        H.push_back(found);
                    }
                } else {
                    boxes_up(found, l);
                    H.at(l + 1) = found;
                }
            } else if (l < top) {
                H.erase(H.begin() + l + 1);
            }
            cells.clear();
        }
        promote();
    }

    void build_hierarchy() {
        determine_maximum();
        H.assign(1, {Box{0, 0, pr.GetXSize(pr.maxDepth), pr.GetPSize(pr.maxDepth)}});
        promote();
        for (int i = 0; i < pr.maxDepth; i++) {
            push_data(1);
            update_hierarchy();
        }
    }

    // ---------------------------------------------------------------- ghost fills
    double same_value(int nb, int gi, int gj, int val) const {  // GetValueFromSameLevel; BC: 0
        if (nb < 0) return 0.0;
        const Patch &N = patches[nb];
        return N.f[val][N.id(gi - N.x_pos, gj - N.p_pos)];
    }
    // Rectangle::GetInterpolantsREF (Rectangle.cpp:121-137)
    static std::vector<double> interp_ref(const Patch &C, double f1, double f2, double f3, double f4, double f5) {
        std::vector<double> t(C.r, 0.0);
        f5 -= f3;
        f4 -= f3;
        f2 -= f3;
        f1 -= f3;
        double a1 = 0.104166666666667 * f1 + -0.708333333333334 * f2 + 0.708333333333334 * f4 + -0.104166666666667 * f5;
        double a2 = 0.117647058823529 * f1 + 0.029411764705882 * f2 + 0.029411764705882 * f4 + 0.117647058823529 * f5;
        double a3 = -0.083333333333333 * f1 + 0.166666666666667 * f2 + -0.166666666666667 * f4 + 0.083333333333334 * f5;
        for (int i = 0; i < C.r; i++) t[i] = C.refc[3 * i] * a1 + C.refc[3 * i + 1] * a2 + C.refc[3 * i + 2] * a3 + f3;
        return t;
    }
    // Rectangle::GetWenoValueFromCoarseLevel (Rectangle.cpp:343-415)
    std::vector<double> weno_coarse(int ci, int gi, int gj, int d, int val) const {
        const Patch &C = patches[ci];
        const int r = C.r;
        const int ic = gi / r - C.x_pos, jc = gj / r - C.p_pos;
        const double *f = C.f[val].data();
        std::vector<std::vector<double>> temps;
        for (int k = -2; k < 3; k++)
            temps.push_back(interp_ref(C, f[C.id(ic - 2, jc + k)], f[C.id(ic - 1, jc + k)], f[C.id(ic, jc + k)],
                                       f[C.id(ic + 1, jc + k)], f[C.id(ic + 2, jc + k)]));
        std::vector<double> it(r * r);
        double sum(0.0);
        for (int k = 0; k < r; k++) {
            auto part = interp_ref(C, temps[0][k], temps[1][k], temps[2][k], temps[3][k], temps[4][k]);
            for (int l = 0; l < r; l++) {
                it[k * r + l] = part[l];
                sum += part[l];
            }
        }
        double correction = f[C.id(ic, jc)] - 1.0 / std::pow(r, 2) * sum;
        for (auto &v : it) v += correction;
        if (d < 0 || d > 3) return it;
        std::vector<double> red(2 * r);
        for (int k = 0; k < r; k++) {
            if (d == 0) red[2 * k] = it[r * k + r - 1], red[2 * k + 1] = it[r * k + r - 2];
            else if (d == 1) red[2 * k] = it[k], red[2 * k + 1] = it[r + k];
            else if (d == 2) red[2 * k] = it[r * k], red[2 * k + 1] = it[r * k + 1];
            else red[2 * k] = it[r * (r - 1) + k], red[2 * k + 1] = it[r * (r - 2) + k];
        }
        return red;
    }
    // Rectangle::UpdateInterriorPoints / GetValueFromFinerLevel (Rectangle.cpp:314-337)
    void update_interior(Patch &R, int val) {
        const int r = R.r;
        for (int i = 0; i < R.nx; i++)
            for (int j = 0; j < R.np; j++)
                if (R.nested[R.id(i, j)]) {
                    const Patch &Fp = patches[R.finer[R.id(i, j)]];
                    const int fi = (R.x_pos + i) * r - Fp.x_pos, fj = (R.p_pos + j) * r - Fp.p_pos;
                    double t(0.0);
                    for (int k = 0; k < r; k++)
                        for (int l = 0; l < r; l++) t += Fp.f[val][Fp.id(fi + k, fj + l)];
                    t /= std::pow((double)r, 2.0);
                    R.f[val][R.id(i, j)] = t;
                }
    }
    // Rectangle::UpdateSameLevelBoundaries (Rectangle.cpp:562-614)
    void update_same(Patch &R, int val) {
        const int r = R.r;
        double *f = R.f[val].data();
        for (size_t e = 0; e + 2 < R.sxm.size(); e++)
            if (R.sxm[e + 1])
                for (int j = 0; j < r; j++) {
                    const int i = (int)e;
                    f[R.id(-1, i * r + j)] = same_value(R.xm[e + 1], R.x_pos - 1, R.p_pos + i * r + j, val);
                    f[R.id(-2, i * r + j)] = same_value(R.xm[e + 1], R.x_pos - 2, R.p_pos + i * r + j, val);
                }
        for (size_t e = 0; e + 2 < R.sxp.size(); e++)
            if (R.sxp[e + 1])
                for (int j = 0; j < r; j++) {
                    const int i = (int)e;
                    f[R.id(R.nx, i * r + j)] = same_value(R.xp[e + 1], R.x_pos + R.nx, R.p_pos + i * r + j, val);
                    f[R.id(R.nx + 1, i * r + j)] = same_value(R.xp[e + 1], R.x_pos + R.nx + 1, R.p_pos + i * r + j, val);
                }
        for (size_t e = 0; e < R.spm.size(); e++)
            if (R.spm[e])
                for (int j = 0; j < r; j++) {
                    const int i = (int)e;
                    f[R.id(i * r + j, -1)] = same_value(R.pm[e], R.x_pos + i * r + j, R.p_pos - 1, val);
                    f[R.id(i * r + j, -2)] = same_value(R.pm[e], R.x_pos + i * r + j, R.p_pos - 2, val);
                }
        for (size_t e = 0; e < R.spp.size(); e++)
            if (R.spp[e])
                for (int j = 0; j < r; j++) {
                    const int i = (int)e;
                    f[R.id(i * r + j, R.np)] = same_value(R.pp[e], R.x_pos + i * r + j, R.p_pos + R.np, val);
                    f[R.id(i * r + j, R.np + 1)] = same_value(R.pp[e], R.x_pos + i * r + j, R.p_pos + R.np + 1, val);
                }
    }
    // Rectangle::UpdateCornerPoints (Rectangle.cpp:1130-1214)
    void update_corners(Patch &R, int val) {
        const int r = R.r;
        double *f = R.f[val].data();
        const int top = (int)R.sxm.size() - 2;
        auto left = [&](int i, int j0, int j1) {
            const int e = i + 1, nb = R.xm[e];
            if (nb >= 0 && !R.sxm[e]) {
                auto t = weno_coarse(nb, R.x_pos - 1, R.p_pos + i * r, 3, val);
                for (int j = j0; j < j1; j++) {
                    f[R.id(-1, i * r + j)] = t[2 * j];
                    f[R.id(-2, i * r + j)] = t[2 * j + 1];
                }
            } else {
                for (int j = j0; j < j1; j++) {
                    f[R.id(-1, i * r + j)] = same_value(nb, R.x_pos - 1, R.p_pos + i * r + j, val);
                    f[R.id(-2, i * r + j)] = same_value(nb, R.x_pos - 2, R.p_pos + i * r + j, val);
                }
            }
        };
        auto right = [&](int i, int j0, int j1) {
            const int e = i + 1, nb = R.xp[e];
            if (nb >= 0 && !R.sxp[e]) {
                auto t = weno_coarse(nb, R.x_pos + R.nx, R.p_pos + i * r, 1, val);
                for (int j = j0; j < j1; j++) {
                    f[R.id(R.nx, i * r + j)] = t[2 * j];
                    f[R.id(R.nx + 1, i * r + j)] = t[2 * j + 1];
                }
            } else {
                for (int j = j0; j < j1; j++) {
                    f[R.id(R.nx, i * r + j)] = same_value(nb, R.x_pos + R.nx, R.p_pos + i * r + j, val);
                    f[R.id(R.nx + 1, i * r + j)] = same_value(nb, R.x_pos + R.nx + 1, R.p_pos + i * r + j, val);
                }
            }
        };
        left(-1, r - 2, r);
        left(top, 0, 2);
        right(-1, r - 2, r);
        right(top, 0, 2);
    }
    // Rectangle::UpdateDifferentLevelBoundaries (Rectangle.cpp:416-560)
    void update_diff(Patch &R, int val) {
        const int r = R.r;
        double *f = R.f[val].data();
        for (size_t e = 0; e + 2 < R.sxm.size(); e++)
            if (!R.sxm[e + 1] && R.xm[e + 1] >= 0) {
                const int i = (int)e;
                auto t = weno_coarse(R.xm[e + 1], R.x_pos - 1, R.p_pos + i * r, 3, val);
                for (int j = 0; j < r; j++) {
                    f[R.id(-1, i * r + j)] = t[2 * j];
                    f[R.id(-2, i * r + j)] = t[2 * j + 1];
                }
            }
        for (size_t e = 0; e + 2 < R.sxp.size(); e++)
            if (!R.sxp[e + 1] && R.xp[e + 1] >= 0) {
                const int i = (int)e;
                auto t = weno_coarse(R.xp[e + 1], R.x_pos + R.nx, R.p_pos + i * r, 1, val);
                for (int j = 0; j < r; j++) {
                    f[R.id(R.nx, i * r + j)] = t[2 * j];
                    f[R.id(R.nx + 1, i * r + j)] = t[2 * j + 1];
                }
            }
        for (size_t e = 0; e < R.spm.size(); e++)
            if (!R.spm[e] && R.pm[e] >= 0) {
                const int i = (int)e;
                auto t = weno_coarse(R.pm[e], R.x_pos + i * r, R.p_pos - 1, 0, val);
                for (int j = 0; j < r; j++) {
                    f[R.id(i * r + j, -1)] = t[2 * j];
                    f[R.id(i * r + j, -2)] = t[2 * j + 1];
                }
            }
        for (size_t e = 0; e < R.spp.size(); e++)
            if (!R.spp[e] && R.pp[e] >= 0) {
                const int i = (int)e;
                auto t = weno_coarse(R.pp[e], R.x_pos + i * r, R.p_pos + R.np, 2, val);
                for (int j = 0; j < r; j++) {
                    f[R.id(i * r + j, R.np)] = t[2 * j];
                    f[R.id(i * r + j, R.np + 1)] = t[2 * j + 1];
                }
            }
        update_corners(R, val);
    }
    // Mesh::PushData (Mesh.cpp:91-106)
    void push_data(int val) {
        const int L = pr.maxDepth + 1;
        for (int k : lv[0]) update_same(patches[k], val);
        for (int i = 1; i < L; i++) {
            for (int k : lv[i]) update_interior(patches[k], val);
            for (int k : lv[i]) update_same(patches[k], val);
        }
        for (int k : lv[L - 1]) update_corners(patches[k], val);
        for (int i = L - 1; i > 0; i--)
            for (int k : lv[i - 1]) update_diff(patches[k], val);
    }

    // ---------------------------------------------------------------- fluxes to coarse
    double gamma_p(const Patch &P, double mom, double as) const { return std::sqrt(1.0 + ((mom * mom) + as) * P.g2); }
    double momentum(const Patch &P, double j) const { return P.pmin + P.dp * (j + P.p_pos); }
    // Rectangle::RGKGetFluxX / RGKGetFluxXL / RGKGetFluxP / RGKGetFluxPL
    // (Rectangle.cpp:1032-1098, 1216-1253) and CalculateFluxToCoarse* (Rectangle.hpp:132-178)
    double rgk_flux(int pi, int i, int j, bool xdir, bool low) const {
        const Patch &P = patches[pi];
        const size_t d = P.id(i, j);
        if (xdir && P.ifx[d]) return flux_to_coarse(P.finer_x[d], P.x_pos + i, P.p_pos + j, true, low);
        if (!xdir && P.ifp[d]) return flux_to_coarse(P.finer_p[d], P.x_pos + i, P.p_pos + j, false, low);
        const double *f = P.f[1].data();
        const double w3 = 1.0 / 48.0;
        const double q = P.q;
        if (xdir) {
            double as = q * q * asq_face(P.rtb * (i + P.x_pos));
            double am = P.dp_inv * P.cc * (gamma_p(P, momentum(P, j + 1), as) - gamma_p(P, momentum(P, j), as));
            if (low) return P.dx_inv * (am > 0.0 ? f[P.id(i - 1, j)] : f[P.id(i, j)]) * am;
            double ap1 = P.dp_inv * P.cc * (gamma_p(P, momentum(P, j + 2.0), as) - gamma_p(P, momentum(P, j + 1.0), as));
            double am1 = P.dp_inv * P.cc * (gamma_p(P, momentum(P, j), as) - gamma_p(P, momentum(P, j - 1.0), as));
            double fm = weno_max(f[P.id(i - 2, j)], f[P.id(i - 1, j)], f[P.id(i, j)], f[P.id(i + 1, j)], am > 0.0);
            double fp1 = weno_max(f[P.id(i - 2, j + 1)], f[P.id(i - 1, j + 1)], f[P.id(i, j + 1)], f[P.id(i + 1, j + 1)], ap1 > 0.0);
            double fm1 = weno_max(f[P.id(i - 2, j - 1)], f[P.id(i - 1, j - 1)], f[P.id(i, j - 1)], f[P.id(i + 1, j - 1)], am1 > 0.0);
            return P.dx_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
        }
        double as_1 = q * q * asq_face(P.rtb * (i + P.x_pos));
        double as_2 = q * q * asq_face(P.rtb * (i + 1 + P.x_pos));
        double Em = q * patch_efield(P, i);
        double mom = momentum(P, j);
        double am = Em - P.cc * P.dx_inv * (gamma_p(P, mom, as_2) - gamma_p(P, mom, as_1));
        if (low) return P.dp_inv * (am > 0.0 ? f[P.id(i, j - 1)] : f[P.id(i, j)]) * am;
        double as_0 = q * q * asq_face(P.rtb * (i - 1 + P.x_pos));
        double as_3 = q * q * asq_face(P.rtb * (i + 2 + P.x_pos));
        double Ep1 = q * patch_efield(P, i + 1), Em1 = q * patch_efield(P, i - 1);
        double ap1 = Ep1 - P.cc * P.dx_inv * (gamma_p(P, mom, as_3) - gamma_p(P, mom, as_2));
        double am1 = Em1 - P.cc * P.dx_inv * (gamma_p(P, mom, as_1) - gamma_p(P, mom, as_0));
        double fm = weno_max(f[P.id(i, j - 2)], f[P.id(i, j - 1)], f[P.id(i, j)], f[P.id(i, j + 1)], am > 0.0);
        double fp1 = weno_max(f[P.id(i + 1, j - 2)], f[P.id(i + 1, j - 1)], f[P.id(i + 1, j)], f[P.id(i + 1, j + 1)], ap1 > 0.0);
        double fm1 = weno_max(f[P.id(i - 1, j - 2)], f[P.id(i - 1, j - 1)], f[P.id(i - 1, j)], f[P.id(i - 1, j + 1)], am1 > 0.0);
        return P.dp_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
    }
    double flux_to_coarse(int fi, int ci, int cj, bool xdir, bool low) const {
        const Patch &Fp = patches[fi];
        const int r = Fp.r;
        const int i = ci * r - Fp.x_pos, j = cj * r - Fp.p_pos;
        double temp = 0.0;
        for (int k = 0; k < r; k++) temp += xdir ? rgk_flux(fi, i, j + k, true, low) : rgk_flux(fi, i + k, j, false, low);
        temp *= (1.0 / (r * r));
        return temp;
    }

    // ---------------------------------------------------------------- limiter exchange
    // Rectangle::SetCFromSameLevel / UpdateCFromSameLevel / SetCFromDifferentLevel
    // (Rectangle.cpp:1625-1960); `N` is the neighbour, `R` the calling patch.
    void c_same(Patch &N, Patch &R, int gi, int gj, int t, bool update) {
        const int in = gi - N.x_pos, jn = gj - N.p_pos, ic = gi - R.x_pos, jc = gj - R.p_pos;
        for (int k = 0; k < N.r; k++) {
            const bool xf = t < 2;
            const size_t dn = xf ? N.id(in, jn + k) : N.id(in + k, jn);
            const size_t dc = xf ? R.id(ic, jc + k) : R.id(ic + k, jc);
            std::vector<double> &NC = xf ? N.Cx : N.Cp, &RC = xf ? R.Cx : R.Cp;
            const std::vector<double> &NDS = xf ? N.FxDS : N.FpDS;
            const size_t np_ = xf ? dn - N.W : dn - 1, cp_ = xf ? dc - R.W : dc - 1;
            double c;
            if (update) c = std::min(NC[dn], RC[dc]);
            else if (t == 0 || t == 2) c = NDS[dn] > 0.0 ? std::min(R.Rp[dc], N.Rm[np_]) : std::min(N.Rp[np_], R.Rm[dc]);
            else c = NDS[dn] > 0.0 ? std::min(R.Rm[cp_], N.Rp[dn]) : std::min(N.Rm[dn], R.Rp[cp_]);
            NC[dn] = c;
            RC[dc] = c;
        }
    }
    void c_diff(Patch &N, Patch &R, int gi, int gj, int t) {
        const int r = N.r;
        const int ic = gi - R.x_pos, jc = gj - R.p_pos;
        const int i0 = gi / r - N.x_pos, j0 = gj / r - N.p_pos;
        const bool xf = t < 2;
        std::vector<double> &NC = xf ? N.Cx : N.Cp, &RC = xf ? R.Cx : R.Cp;
        const std::vector<double> &NDS = xf ? N.FxDS : N.FpDS, &RDS = xf ? R.FxDS : R.FpDS;
        const size_t dn = N.id(i0, j0), np_ = xf ? N.id(i0 - 1, j0) : N.id(i0, j0 - 1);
        double c = NC[dn];
        for (int k = 0; k < r; k++) {
            const size_t dc = xf ? R.id(ic, jc + k) : R.id(ic + k, jc);
            const size_t cp_ = xf ? R.id(ic - 1, jc + k) : R.id(ic + k, jc - 1);
            if (t == 0 || t == 2) c = std::min(c, RDS[dc] > 0.0 ? R.Rp[dc] : R.Rm[dc]);
            else c = std::min(c, RDS[dc] > 0.0 ? R.Rm[cp_] : R.Rp[cp_]);
        }
        if (t == 0 || t == 2) c = std::min(c, NDS[dn] > 0.0 ? N.Rm[np_] : N.Rp[np_]);
        else c = std::min(c, NDS[dn] > 0.0 ? N.Rp[dn] : N.Rm[dn]);
        for (int k = 0; k < r; k++) RC[xf ? R.id(ic, jc + k) : R.id(ic + k, jc)] = c;
        NC[dn] = c;
    }
    // CalculateSameBoundaryC / CalculateDifferentBoundaryC / UpdateSameBoundaryC of one
    // patch (kind 0 / 1 / 2); the domain boundary object does nothing.
    void c_calls(int ri, int kind) {
        Patch &R = patches[ri];
        const int r = R.r;
        auto one = [&](int nb, bool same, int gi, int gj, int t) {
            if (nb < 0) return;
            if (kind == 1) {
                if (!same) c_diff(patches[nb], R, gi, gj, t);
            } else if (same) {
                c_same(patches[nb], R, gi, gj, t, kind == 2);
            }
        };
        for (size_t e = 0; e + 2 < R.sxm.size(); e++) one(R.xm[e + 1], R.sxm[e + 1], R.x_pos, R.p_pos + (int)e * r, 0);
        for (size_t e = 0; e + 2 < R.sxp.size(); e++) one(R.xp[e + 1], R.sxp[e + 1], R.x_pos + R.nx, R.p_pos + (int)e * r, 1);
        for (size_t e = 0; e < R.spm.size(); e++) one(R.pm[e], R.spm[e], R.x_pos + (int)e * r, R.p_pos, 2);
        for (size_t e = 0; e < R.spp.size(); e++) one(R.pp[e], R.spp[e], R.x_pos + (int)e * r, R.p_pos + R.np, 3);
    }
    // Mesh::PushBoundaryC (Mesh.cpp:904-917)
    void push_boundary_c() {
        for (int kind = 0; kind < 3; kind++)
            for (int l = 0; l <= pr.maxDepth; l++)
                for (int k : lv[l]) c_calls(k, kind);
    }

    // ---------------------------------------------------------------- moments
    double rel_value(const Patch &P, int i, int j, int k) const {
        const double *f = P.f[1].data();
        const double f3 = f[P.id(i, j)];
        if (P.rtb == 1) return f3;
        double g1 = f[P.id(i - 2, j)] - f3, g2 = f[P.id(i - 1, j)] - f3;
        double g4 = f[P.id(i + 1, j)] - f3, g5 = f[P.id(i + 2, j)] - f3;
        double a1 = 0.104166666666667 * g1 + -0.708333333333334 * g2 + 0.708333333333334 * g4 + -0.104166666666667 * g5;
        double a2 = 0.117647058823529 * g1 + 0.029411764705882 * g2 + 0.029411764705882 * g4 + 0.117647058823529 * g5;
        double a3 = -0.083333333333333 * g1 + 0.166666666666667 * g2 + -0.166666666666667 * g4 + 0.083333333333334 * g5;
        double te = 0.0, mine = 0.0;
        for (int q = 0; q < P.rtb; q++) {
            double v = P.relc[3 * q] * a1 + P.relc[3 * q + 1] * a2 + P.relc[3 * q + 2] * a3 + f3;
            te += v;
            if (q == k) mine = v;
        }
        double cor = f3 - (1.0 / (double)P.rtb) * te;
        return mine + cor;
    }

    void moments(Patch &P) {
        const double q = P.q, mass = P.m;
        const double c1 = (1 / mass) * c_inv, c2 = 1 / c1, c3 = 1 / 48.0;
        const int rtb = P.rtb;
#pragma omp parallel for schedule(guided)
        for (int i = 0; i < P.nx; i++) {
            for (int k = 0; k < rtb; k++) {
                const double a = (q * q) * cell_asq((i + P.x_pos) * rtb + k);
                std::vector<double> Lr(P.np + 2);
                for (int j = -1; j <= P.np; j++) {
                    double p0 = P.pmin + P.dp * (double)(j + P.p_pos);
                    double p1 = P.pmin + P.dp * (double)(j + 1 + P.p_pos);
                    double g0 = std::sqrt(1.0 + ((p0 * p0) + a) * P.g2);
                    double g1 = std::sqrt(1.0 + ((p1 * p1) + a) * P.g2);
                    Lr[j + 1] = c2 * std::log((g1 + c1 * p1) / (g0 + c1 * p0));
                }
                double vm1 = rel_value(P, i, -1, k), v0 = rel_value(P, i, 0, k), vp1 = rel_value(P, i, 1, k);
                double ch = 0.0, cu = 0.0;
                for (int j = 0; j < P.np; j++) {
                    if (!P.nested[P.id(i, j)]) {
                        ch += v0;
                        double gm = Lr[j + 1], gm1 = Lr[j], gp1 = Lr[j + 2];
                        cu += v0 * gm + c3 * (gp1 - gm1) * (vp1 - vm1);
                    }
                    vm1 = v0;
                    v0 = vp1;
                    vp1 = rel_value(P, i, j + 2, k);
                }
                P.chargeR[i * rtb + k] = ch * (P.dp * q);
                P.currentR[i * rtb + k] = cu * (-q * q / mass);
            }
        }
    }

    // Level::CollectRhoAndJ + EMFieldSolver::AssembleRhoAndJ (Level.cpp:19-62,
    // EMSolver.cpp:104-122): per level, patch sums in level order; levels finest first.
    void assemble() {
        for (auto &P : patches) moments(P);
        for (int x = 0; x < F.n; x++) {
            double J = 0.0, charge = 0.0, cs_ = 0.0;
            for (int l = 0; l <= pr.maxDepth; l++) {
                double lc = 0.0, lj = 0.0;
                for (int k : lv[l]) {
                    const Patch &P = patches[k];
                    int c = x - P.x_pos * P.rtb;
                    if (c >= 0 && c < P.nx * P.rtb) {
                        lc += P.chargeR[c];
                        lj += P.currentR[c];
                    }
                }
                cs_ += lc;
                J += lj;
            }
            charge += cs_;
            F.charge[x] = charge;
            F.J[x] = J;
        }
    }

    void poisson() {
        const int n = F.n;
        const double w = std::pow(pr.GetDx(0), 2.0);
        for (int i = 0; i < n; i++) F.phi[i] = eps0_inv * (F.charge[i] + F.neut[i]);
        for (int i = 0; i < n; i++) F.phi[i] *= w;
        lu.solve(F.phi.data());
        F.Ex0 += -(efield(-1) + efield(0)) * 0.5;
    }

    // ---------------------------------------------------------------- FCT sub-steps
    void fct_sub0(int pi, int step, const double *a, double asum) {
        Patch &P = patches[pi];
        const int nx = P.nx, np = P.np;
        const double *f = P.f[1].data();
        const double w3 = 1 / 48.0;
#pragma omp parallel for schedule(guided)
        for (int i = -1; i <= nx + 1; i++) {
            double as = P.q * P.q * asq_face(P.rtb * (i + P.x_pos));
            for (int j = -1; j <= np + 1; j++) {
                double p = P.pmin + P.dp * (double)(j + P.p_pos);
                P.gam[P.id(i, j)] = std::sqrt(1.0 + ((p * p) + as) * P.g2);
            }
        }
#pragma omp parallel for schedule(guided)
        for (int i = -1; i <= nx; i++) {
            double Em = P.q * patch_efield(P, i);
            for (int j = -1; j <= np; j++) {
                if (i >= 0) {
                    double am = P.dp_inv * P.cc * (P.gam[P.id(i, j + 1)] - P.gam[P.id(i, j)]);
                    P.ex[P.id(i, j)] = am;
                    P.fx[P.id(i, j)] = weno(f[P.id(i - 2, j)], f[P.id(i - 1, j)], f[P.id(i, j)], f[P.id(i + 1, j)], am > 0.0);
                }
                if (j >= 0) {
                    double am = Em - P.cc * P.dx_inv * (P.gam[P.id(i + 1, j)] - P.gam[P.id(i, j)]);
                    P.ep[P.id(i, j)] = am;
                    P.fp[P.id(i, j)] = weno(f[P.id(i, j - 2)], f[P.id(i, j - 1)], f[P.id(i, j)], f[P.id(i, j + 1)], am > 0.0);
                }
            }
        }
#pragma omp parallel for schedule(guided)
        for (int i = -1; i <= nx; i++) {
            for (int j = -1; j <= np; j++) {
                size_t d = P.id(i, j);
                if (i >= 0 && P.ifx[d]) {  // coarse/fine interface: the finer patch's mean flux
                    P.FxH[step][d] = flux_to_coarse(P.finer_x[d], P.x_pos + i, P.p_pos + j, true, false);
                    if (step == 0) P.FxL[d] = flux_to_coarse(P.finer_x[d], P.x_pos + i, P.p_pos + j, true, true);
                } else if (i >= 0) {
                    double am = P.ex[d], ap1 = P.ex[d + 1], am1 = P.ex[d - 1];
                    double fm = P.fx[d], fp1 = P.fx[d + 1], fm1 = P.fx[d - 1];
                    P.FxH[step][d] = P.dx_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
                    if (step == 0) P.FxL[d] = P.dx_inv * ((am > 0.0 ? f[d - P.W] : f[d]) * am);
                }
                if (j >= 0 && P.ifp[d]) {
                    P.FpH[step][d] = flux_to_coarse(P.finer_p[d], P.x_pos + i, P.p_pos + j, false, false);
                    if (step == 0) P.FpL[d] = flux_to_coarse(P.finer_p[d], P.x_pos + i, P.p_pos + j, false, true);
                } else if (j >= 0) {
                    double am = P.ep[d], ap1 = P.ep[d + P.W], am1 = P.ep[d - P.W];
                    double fm = P.fp[d], fp1 = P.fp[d + P.W], fm1 = P.fp[d - P.W];
                    P.FpH[step][d] = P.dp_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
                    if (step == 0) P.FpL[d] = P.dp_inv * ((am > 0.0 ? f[d - 1] : f[d]) * am);
                }
            }
        }
        const int xm = P.left ? 1 : 0, xp = P.right ? nx : nx + 1, pm = P.down ? 1 : 0, pp = P.up ? np : np + 1;
        auto act = [&](int i, int j) { return i >= xm && i < xp && j >= pm && j < pp; };
#pragma omp parallel for schedule(guided)
        for (int i = -2; i <= nx + 1; i++) {
            for (int j = -2; j <= np + 1; j++) {
                size_t d = P.id(i, j);
                double hx = a[0] * P.FxH[0][d], hp = a[0] * P.FpH[0][d];
                for (int k = 1; k <= step; k++) {
                    if (step == 5 && k == 1) continue;
                    hx = hx + a[k] * P.FxH[k][d];
                    hp = hp + a[k] * P.FpH[k][d];
                }
                double lsx = asum * P.FxL[d], lsp = asum * P.FpL[d];
                P.FxDS[d] = hx - lsx;
                P.FpDS[d] = hp - lsp;
            }
        }
        double *f2 = P.f[2].data();
        const double *f0 = P.f[0].data();
#pragma omp parallel for schedule(guided)
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < np; j++) {
                size_t d = P.id(i, j);
                double v = f0[d];
                if (act(i, j)) v += asum * P.FxL[d];
                if (act(i, j)) v += asum * P.FpL[d];
                if (act(i, j + 1)) v -= asum * P.FpL[d + 1];
                if (act(i + 1, j)) v -= asum * P.FxL[d + P.W];
                f2[d] = v;
            }
    }

    void fct_sub1(Patch &P) {
        const int nx = P.nx, np = P.np, W = P.W;
        const double *f0 = P.f[0].data(), *f2 = P.f[2].data();
#pragma omp parallel for schedule(guided)
        for (int i = -1; i <= nx; i++)
            for (int j = -1; j <= np; j++) {
                size_t d = P.id(i, j);
                double dxi = P.FxDS[d], dxn = P.FxDS[d + W], dpi = P.FpDS[d], dpn = P.FpDS[d + 1];
                double Pp = vmax(0.0, dxi) - vmin(0.0, dxn) + vmax(0.0, dpi) - vmin(0.0, dpn);
                double Pm = vmax(0.0, dxn) - vmin(0.0, dxi) + vmax(0.0, dpn) - vmin(0.0, dpi);
                double wMax = vmax(vmax(f0[d], f2[d]), vmax(vmax(f0[d + W], f2[d + W]),
                                   vmax(vmax(f0[d - W], f2[d - W]), vmax(vmax(f0[d + 1], f2[d + 1]), vmax(f0[d - 1], f2[d - 1])))));
                double wMin = vmin(vmin(f0[d], f2[d]), vmin(vmin(f0[d + W], f2[d + W]),
                                   vmin(vmin(f0[d - W], f2[d - W]), vmin(vmin(f0[d + 1], f2[d + 1]), vmin(f0[d - 1], f2[d - 1])))));
                double Qm = -wMin + f2[d], Qp = wMax - f2[d];
                P.Rp[d] = Pp > 0.0 ? vmin(1.0, Qp / Pp) : 0.0;
                P.Rm[d] = Pm > 0.0 ? vmin(1.0, Qm / Pm) : 0.0;
            }
        std::fill(P.Cx.begin(), P.Cx.end(), 1.0);
        std::fill(P.Cp.begin(), P.Cp.end(), 1.0);
#pragma omp parallel for schedule(guided)
        for (int i = 1; i < nx; i++)
            for (int j = 0; j < np; j++) {
                size_t d = P.id(i, j);
                P.Cx[d] = P.FxDS[d] > 0.0 ? vmin(P.Rp[d], P.Rm[d - W]) : vmin(P.Rp[d - W], P.Rm[d]);
                P.Cp[d] = P.FpDS[d] > 0.0 ? vmin(P.Rp[d], P.Rm[d - 1]) : vmin(P.Rp[d - 1], P.Rm[d]);
            }
    }

    void fct_sub2(Patch &P) {
        const int nx = P.nx, np = P.np, W = P.W;
        const int xm = P.left ? 1 : 0, xp = P.right ? nx : nx + 1, pm = P.down ? 1 : 0, pp = P.up ? np : np + 1;
        auto act = [&](int i, int j) { return i >= xm && i < xp && j >= pm && j < pp; };
        double *f1 = P.f[1].data();
        const double *f2 = P.f[2].data();
#pragma omp parallel for schedule(guided)
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < np; j++) {
                size_t d = P.id(i, j);
                double v = f2[d];
                if (act(i, j)) v += P.Cx[d] * P.FxDS[d];
                if (act(i, j)) v += P.Cp[d] * P.FpDS[d];
                if (act(i, j + 1)) v -= P.Cp[d + 1] * P.FpDS[d + 1];
                if (act(i + 1, j)) v -= P.Cx[d + W] * P.FxDS[d + W];
                f1[d] = v;
            }
    }

    // ---------------------------------------------------------------- Maxwell
    void maxwell(int step, double timestep) {
        const int nf = F.nf, pre = F.pre, n = F.n;
        const double dx_inv = 1 / pr.GetDx(0);
        const double bz0 = pr.BZ(0, time), by0 = pr.BY(0, time);
        auto S1 = [&](std::vector<double> &X, int i) { return X[F.I(i, 1)]; };
        for (int i = 0; i < nf; i++) {
            double rBy = 0, rBz = 0, rEy = 0, rEz = 0, rAy = 0, rAz = 0;
            if (i == 0) {
                rBy = dx_inv * (S1(F.Ez, 1) - S1(F.Ez, 0));
                rBz = -dx_inv * (S1(F.Ey, 1) - S1(F.Ey, 0));
                rEy = -dx_inv * (S1(F.Bz, 0) - bz0) * eps0_inv * mu_inv;
                rEz = dx_inv * (S1(F.By, 0) - by0) * eps0_inv * mu_inv;
                rAy = -S1(F.Ey, 0);
                rAz = -S1(F.Ez, 0);
            } else if (i < pre || (i >= pre + n && i < nf - 2)) {
                rBy = dx_inv * (S1(F.Ez, i + 1) - S1(F.Ez, i));
                rBz = -dx_inv * (S1(F.Ey, i + 1) - S1(F.Ey, i));
                rEy = -dx_inv * (S1(F.Bz, i) - S1(F.Bz, i - 1)) * eps0_inv * mu_inv;
                rEz = dx_inv * (S1(F.By, i) - S1(F.By, i - 1)) * eps0_inv * mu_inv;
                rAy = -S1(F.Ey, i);
                rAz = -S1(F.Ez, i);
            } else if (i >= pre && i < pre + n) {
                const double c1 = -1.0 / 24, c2 = 9.0 / 8.0;
                const double Jv = F.J[i - pre];
                rBy = dx_inv * (c1 * (S1(F.Ez, i + 2) - S1(F.Ez, i - 1)) + c2 * (S1(F.Ez, i + 1) - S1(F.Ez, i)));
                rBz = -dx_inv * (c1 * (S1(F.Ey, i + 2) - S1(F.Ey, i - 1)) + c2 * (S1(F.Ey, i + 1) - S1(F.Ey, i)));
                rEy = -dx_inv * (c1 * (S1(F.Bz, i + 1) - S1(F.Bz, i - 2)) + c2 * (S1(F.Bz, i) - S1(F.Bz, i - 1))) * eps0_inv * mu_inv -
                      eps0_inv * Jv * S1(F.Ay, i);
                rEz = dx_inv * (c1 * (S1(F.By, i + 1) - S1(F.By, i - 2)) + c2 * (S1(F.By, i) - S1(F.By, i - 1))) * eps0_inv * mu_inv -
                      eps0_inv * Jv * S1(F.Az, i);
                rAy = -S1(F.Ey, i);
                rAz = -S1(F.Ez, i);
            }
            const int s2 = step + 2;
            F.By[F.I(i, s2)] = rBy;
            F.Bz[F.I(i, s2)] = rBz;
            F.Ey[F.I(i, s2)] = rEy;
            F.Ez[F.I(i, s2)] = rEz;
            F.Ay[F.I(i, s2)] = rAy;
            F.Az[F.I(i, s2)] = rAz;
        }
        double c[6] = {0, 0, 0, 0, 0, 0};
        static const double R[6][6] = {
            {0.5, 0, 0, 0, 0, 0},
            {0.221776, 0.110224, 0, 0, 0, 0},
            {-0.04884659515311857, -0.17772065232640102, 0.8465672474795197, 0, 0, 0},
            {-0.15541685842491548, -0.3567050098221991, 1.0587258798684427, 0.30339598837867193, 0, 0},
            {0.2014243506726763, 0.008742057842904185, 0.15993995707168115, 0.4038290605220775, 0.22606457389066084, 0},
            {0.15791629516167136, 0.0, 0.18675894052400077, 0.6805652953093346, -0.27524053099500667, 0.25}};
        if (step < 5) {
            for (int k = 0; k <= step; k++) c[k] = R[step][k] * timestep;
        } else {
            double a[6];
            for (int k = 0; k < 5; k++) a[k] = R[4][k] * timestep;
            a[5] = 0;
            for (int k = 0; k < 6; k++) c[k] = R[5][k] * timestep - a[k];
        }
        for (auto *Xp : {&F.By, &F.Bz, &F.Ey, &F.Ez, &F.Ay, &F.Az}) {
            auto &X = *Xp;
            for (int i = 0; i < nf; i++) {
                if (step < 5) {
                    double v = X[F.I(i, 0)] + c[0] * X[F.I(i, 2)];
                    for (int k = 1; k <= step; k++) v = v + c[k] * X[F.I(i, k + 2)];
                    X[F.I(i, 1)] = v;
                } else {
                    double v = X[F.I(i, 1)] + c[0] * X[F.I(i, 2)];
                    for (int k = 1; k <= 5; k++) v = v + c[k] * X[F.I(i, k + 2)];
                    X[F.I(i, 0)] = v;
                    X[F.I(i, 1)] = v;
                }
            }
        }
        for (int i = 0; i < n; i++) {
            const double *Ay = &F.Ay[F.I(pre + i, 1)], *Az = &F.Az[F.I(pre + i, 1)];
            double a_y = face_a(Ay[-2], Ay[-1], Ay[0], Ay[1]);
            double a_z = face_a(Az[-2], Az[-1], Az[0], Az[1]);
            F.asq[i] = (a_y * a_y) + (a_z * a_z);
        }
    }

    void update_time(int step, double dt) {
        if (step == 1) time += (0.5 * dt);
        else if (step == 2) time += (0.332 - 0.5) * dt;
        else if (step == 3) time += (0.62 - 0.332) * dt;
        else if (step == 4) time += (0.85 - 0.62) * dt;
        else if (step == 5) time += (1.0 - 0.85) * dt;
    }

    void advance(double timestep) {
        static const double R[6][6] = {
            {0.5, 0, 0, 0, 0, 0},
            {0.221776, 0.110224, 0, 0, 0, 0},
            {-0.04884659515311857, -0.17772065232640102, 0.8465672474795197, 0, 0, 0},
            {-0.15541685842491548, -0.3567050098221991, 1.0587258798684427, 0.30339598837867193, 0, 0},
            {0.2014243506726763, 0.008742057842904185, 0.15993995707168115, 0.4038290605220775, 0.22606457389066084, 0},
            {0.15791629516167136, 0.0, 0.18675894052400077, 0.6805652953093346, -0.27524053099500667, 0.25}};
        for (int s = 0; s < 6; s++) {
            assemble();
            poisson();
            double a[6] = {0, 0, 0, 0, 0, 0};
            const int kmax = s;
            for (int k = 0; k <= kmax; k++) a[k] = R[s][k] * timestep;
            double asum = a[0];
            for (int k = 1; k <= kmax; k++) asum = asum + a[k];
            // Mesh::Advance (Mesh.cpp:64-89): each sub-step over the levels coarsest first
            const int L = pr.maxDepth + 1;
            for (int l = L - 1; l > -1; l--)
                for (int k : lv[l]) fct_sub0(k, s, a, asum);
            push_data(2);
            for (int l = L - 1; l > -1; l--)
                for (int k : lv[l]) fct_sub1(patches[k]);
            push_boundary_c();
            for (int l = L - 1; l > -1; l--)
                for (int k : lv[l]) fct_sub2(patches[k]);
            push_data(1);
            if (s == 5)
                for (auto &P : patches) P.f[0] = P.f[1];
            update_time(s, timestep);
            maxwell(s, timestep);
        }
    }

    double calculate_dt() {
        const double dps = 1 / pr.GetDp(0);
        const double dpsMax = std::max(0.0, std::fabs(pr.q) * dps);
        double pc = 0.0;
        for (int i = 0; i < F.n; i++) {
            double Azv = F.Az[i], Ayv = F.Ay[i];
            double As = Ayv * Ayv + Azv * Azv;
            double temp = 0.0;
            temp = std::max(temp, std::fabs(pr.q) / pr.m / std::sqrt(1 + As / ((pr.m * cs) * (pr.m * cs))) * dps);
            pc = std::max(pc, temp * std::fabs(Ayv * F.Bz[i] - Azv * F.By[i]) + dpsMax * std::fabs(efield(i)));
        }
        return P_cfl() * (1.0 / std::max((cs / pr.GetDx(0) + pc), 1e-40));
    }
    double P_cfl() const { return pr.P.cfl; }

    // ---------------------------------------------------------------- state files
    void write_state(const std::string &path, double dt, long long step) {
        FILE *fp = fopen(path.c_str(), "wb");
        if (!fp) {
            perror(path.c_str());
            exit(2);
        }
        auto wi = [&](long long v) { fwrite(&v, 8, 1, fp); };
        auto wd = [&](double v) { fwrite(&v, 8, 1, fp); };
        auto wv = [&](const std::vector<double> &v) {
            wi((long long)v.size());
            fwrite(v.data(), 8, v.size(), fp);
        };
        fwrite("VXST0001", 1, 8, fp);
        wi(step);
        wd(time);
        wd(dt);
        wd(F.Ex0);
        wi(F.n);
        wi(F.pre);
        wi(F.post);
        for (auto *v : {&F.By, &F.Bz, &F.Ey, &F.Ez, &F.Ay, &F.Az, &F.asq, &F.phi, &F.charge, &F.J, &F.neut}) wv(*v);
        wi(1);  // species
        wi(pr.maxDepth + 1);
        for (int l = 0; l <= pr.maxDepth; l++) {
            wi((long long)lv[l].size());
            for (int k : lv[l]) {
                const Patch &P = patches[k];
                for (long long v : {(long long)P.x_pos, (long long)P.p_pos, (long long)P.nx, (long long)P.np,
                                    (long long)P.depth, (long long)P.up, (long long)P.down, (long long)P.left,
                                    (long long)P.right})
                    wi(v);
                std::vector<double> fv((size_t)3 * (P.nx + 4) * P.W);
                for (size_t c = 0; c < (size_t)(P.nx + 4) * P.W; c++)
                    for (int s = 0; s < 3; s++) fv[3 * c + s] = P.f[s][c];
                wv(fv);
            }
        }
        fclose(fp);
    }

    void read_state(const std::string &path) {
        FILE *fp = fopen(path.c_str(), "rb");
        if (!fp) {
            perror(path.c_str());
            exit(2);
        }
        auto need = [&](void *p, size_t n) {
            if (fread(p, 1, n, fp) != n) {
                fprintf(stderr, "truncated state\n");
                exit(2);
            }
        };
        auto ri = [&]() {
            long long v;
            need(&v, 8);
            return v;
        };
        auto rd = [&]() {
            double v;
            need(&v, 8);
            return v;
        };
        auto rv = [&](std::vector<double> &v) {
            long long n = ri();
            if ((size_t)n != v.size()) {
                fprintf(stderr, "state size mismatch\n");
                exit(2);
            }
            need(v.data(), 8 * v.size());
        };
        char magic[8];
        need(magic, 8);
        ri();
        time = rd();
        rd();
        F.Ex0 = rd();
        if (ri() != F.n || ri() != F.pre || ri() != F.post) {
            fprintf(stderr, "grid mismatch\n");
            exit(2);
        }
        for (auto *v : {&F.By, &F.Bz, &F.Ey, &F.Ez, &F.Ay, &F.Az, &F.asq, &F.phi, &F.charge, &F.J, &F.neut}) rv(*v);
        if (ri() != 1) {
            fprintf(stderr, "the port handles one species\n");
            exit(3);
        }
        long long nl = ri();
        if (nl != pr.maxDepth + 1) {
            fprintf(stderr, "level count mismatch\n");
            exit(2);
        }
        patches.clear();
        lv.assign(nl, {});
        for (long long l = 0; l < nl; l++) {
            long long nr = ri();
            for (long long k = 0; k < nr; k++) {
                long long h[9];
                for (auto &x : h) x = ri();
                if (h[4] != l) {
                    fprintf(stderr, "patch depth mismatch\n");
                    exit(2);
                }
                Patch P = make_patch((int)h[4], (int)h[0], (int)h[1], (int)h[2], (int)h[3]);
                P.up = h[5];
                P.down = h[6];
                P.left = h[7];
                P.right = h[8];
                std::vector<double> fv((size_t)3 * (P.nx + 4) * P.W);
                rv(fv);
                for (size_t c = 0; c < (size_t)(P.nx + 4) * P.W; c++)
                    for (int s = 0; s < 3; s++) P.f[s][c] = fv[3 * c + s];
                lv[l].push_back((int)patches.size());
                patches.push_back(std::move(P));
            }
        }
        connect_keep_f();
        fclose(fp);
    }
};

}  // namespace

int main(int argc, char **argv) {
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto eq = a.find('=');
        if (eq == std::string::npos) {
            fprintf(stderr, "bad argument %s\n", a.c_str());
            return 2;
        }
        kv[a.substr(0, eq)] = a.substr(eq + 1);
    }
    auto getd = [&](const char *k, double d) { return kv.count(k) ? std::stod(kv[k]) : d; };
    auto geti = [&](const char *k, long long d) { return kv.count(k) ? std::stoll(kv[k]) : d; };
    Solver S;
    Params &P = S.pr.P;
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
    P.bdens = getd("bdens", P.bdens);
    P.bp0 = getd("bp0", P.bp0);
    P.bTe = getd("bTe", P.bTe);
    long long steps = geti("steps", 0), dump_every = geti("dump_every", 0), time_steps = geti("time_steps", 0);
    std::string dumpdir = kv.count("dumpdir") ? kv["dumpdir"] : "";
    std::vector<double> dts;
    if (kv.count("dts")) {
        std::stringstream ss(kv["dts"]);
        std::string tok;
        while (std::getline(ss, tok, ',')) dts.push_back(std::stod(tok));
    }
    S.setup();
    auto t0 = std::chrono::steady_clock::now();
    if (kv.count("load")) S.read_state(kv["load"]);
    else S.init_distribution();
    auto t1 = std::chrono::steady_clock::now();
    char name[512];
    if (!dumpdir.empty()) {
        snprintf(name, sizeof name, "%s/state_%05lld.bin", dumpdir.c_str(), 0LL);
        S.write_state(name, 0.0, 0);
    }
    for (long long s = 1; s <= steps; s++) {
        double dt = (s - 1 < (long long)dts.size()) ? dts[s - 1] : S.calculate_dt();
        S.advance(dt);
        if (!dumpdir.empty() && dump_every > 0 && s % dump_every == 0) {
            snprintf(name, sizeof name, "%s/state_%05lld.bin", dumpdir.c_str(), s);
            S.write_state(name, dt, s);
        }
    }
    if (time_steps > 0) {
        const long long warmup = std::max(1LL, geti("warmup", 1));
        for (long long w = 0; w < warmup; w++) S.advance(S.calculate_dt());
        std::vector<double> per;
        for (long long s = 0; s < time_steps; s++) {
            double dt = S.calculate_dt();
            auto a = std::chrono::steady_clock::now();
            S.advance(dt);
            auto b = std::chrono::steady_clock::now();
            per.push_back(std::chrono::duration<double>(b - a).count());
        }
        std::sort(per.begin(), per.end());
        long long cells = 0;
        for (auto &p : S.patches) cells += (long long)p.nx * p.np;  // every level, covered cells included
        printf("{\"cells\": %lld, \"patches\": %zu, \"steps\": %lld, \"best_s\": %.6f, \"median_s\": %.6f, "
               "\"threads\": %d, \"init_s\": %.3f}\n",
               cells, S.patches.size(), time_steps, per.front(), per[per.size() / 2], omp_get_max_threads(),
               std::chrono::duration<double>(t1 - t0).count());
    }
    return 0;
}
