// Diagnostics in the reference's text formats, so its viewer and post-processing read
// the GPU runs: SolverManager::fileOutput (SolverManager.cpp:101-159) with the
// EMFieldSolver dump routines (EMSolver.cpp:340-477) and Mesh::outputRectangleData
// (Mesh.cpp:877-902).
//
// Each file of a run is created by the run's first write and appended to afterwards (the
// reference opens its streams on the first dump and keeps them).  Values are the run's
// own: the species charges are assembled on the host from the patches' moment columns
// in the reference's order (Level::CollectRhoAndJ, EMFieldSolver::AssembleRhoAndJ), the
// momentum spectra dN/dp are formed from f slot 1 as Rectangle::CalculateEnergy does,
// sequentially in x (the reference's OpenMP loop over x accumulates into shared bins), and
// the fields are copied from the device.  Host arithmetic is unfused (-ffp-contract=off),
// so an FP64 run's files match the reference build's text.
#include <cmath>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <stdexcept>

#include "../../include/vx.h"
#include "engine.hpp"

namespace vx {

namespace {

// Rectangle::GetInterpolantsREL's weights for rtb sub-cells (Rectangle.cpp:94-110).
std::vector<double> rel_weights(int rtb) {
    std::vector<double> w;
    const double rb = rtb;
    for (int i = 0; i < rtb; i++) {
        double tl = -0.5 + i / rb;
        double tr = -0.5 + (i + 1.0) / rb;
        w.push_back((tl + tr) * 0.5);
        w.push_back((tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12));
        w.push_back((tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25);
    }
    return w;
}

template <class T>
std::vector<T> to_host(const T *d, size_t n, cudaStream_t st) {
    std::vector<T> h(n);
    if (n) VX_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, st));
    VX_CUDA(cudaStreamSynchronize(st));
    return h;
}

}  // namespace

std::ofstream &Run::out_stream(const std::string &path, int digits) {
    auto it = out_streams.find(path);
    if (it != out_streams.end()) return *it->second;
    auto s = std::make_unique<std::ofstream>(path);
    if (!*s) throw std::runtime_error("cannot open " + path);
    (*s) << std::scientific << std::setprecision(digits);
    return *(out_streams[path] = std::move(s));
}

// f of a patch's slot (0 or 1) as doubles over the padded block, row pitch `pitch`
// (FP32 runs: the stored value divided back by fnorm).
std::vector<double> Run::slot_to_host(const Rect &r, int slot) {
    const size_t pe = r.plane_elems();
    const void *src = slot == 0 ? r.desc.f0 : r.desc.f1;
    std::vector<double> h(pe);
    if (r.esize == 8) {
        VX_CUDA(cudaMemcpyAsync(h.data(), src, pe * sizeof(double), cudaMemcpyDeviceToHost, eng->stream));
        VX_CUDA(cudaStreamSynchronize(eng->stream));
    } else {
        auto f = to_host((const float *)src, pe, eng->stream);
        const double inv = 1.0 / fnorm[r.species];
        for (size_t q = 0; q < pe; q++) h[q] = (double)f[q] * inv;
    }
    return h;
}

void Run::write_fields(const std::string &dir, unsigned mask, int digits, double t) {
    const Settings &s = *S;
    eng->sync();
    const std::string d = dir.empty() ? std::string(".") : dir;
    auto line = [](std::ofstream &o, const double *v, size_t n) {
        for (size_t i = 0; i < n; i++) o << v[i] << " ";
        o << std::endl;
    };
    if (mask & VX_OUT_CHARGE) {  // charge.txt: one line per species (EMSolver.cpp:340-358)
        std::ofstream &o = out_stream(d + "/charge.txt", digits);
        for (size_t sp = 0; sp < rects.size(); sp++) {
            std::vector<double> charges(n, 0.0);
            for (auto &lvl : rects[sp]) {  // coarsest level first (Mesh::InterpolateRhoAndJToFinestMesh)
                std::vector<double> chargeL(n, 0.0);
                for (auto &rp : lvl) {  // Level::CollectRhoAndJ
                    const Rect &r = *rp;
                    const int rtb = r.desc.rtb;
                    const size_t nc = (size_t)r.n_x * rtb;
                    std::vector<double> col(nc);
                    if (precision == kF32) {  // FP32 pairs of the column sums, then their scale
                        auto pr = to_host((const float *)r.desc.chargeR, 2 * nc, eng->stream);
                        for (size_t c = 0; c < nc; c++)
                            col[c] = ((double)pr[2 * c] + (double)pr[2 * c + 1]) * r.desc.msc_rho;
                    } else {
                        col = to_host(r.desc.chargeR, nc, eng->stream);
                    }
                    const size_t shift = (size_t)r.x_pos * rtb;
                    for (size_t c = 0; c < nc; c++) chargeL[shift + c] += col[c];
                }
                for (int i = 0; i < n; i++) charges[i] += chargeL[i];
            }
            line(o, charges.data(), charges.size());
        }
    }
    if (mask & VX_OUT_ENERGY) {  // dNdP_<species>.txt (EMSolver.cpp:361-378, Rectangle.cpp:284-305)
        for (size_t sp = 0; sp < rects.size(); sp++) {
            std::vector<double> energy(s.p_size_finest[sp], 0.0);
            for (auto &lvl : rects[sp]) {
                std::vector<double> energyL(s.p_size_finest[sp], 0.0);
                for (auto &rp : lvl) {
                    const Rect &r = *rp;
                    const int rtb = r.desc.rtb, pit = r.pitch;
                    const std::vector<double> w = rel_weights(rtb);
                    const double m0 = 0.104166666666667, m1 = -0.708333333333334, m2 = 0.708333333333334,
                                 m3 = -0.104166666666667;
                    const double m4 = 0.117647058823529, m5 = 0.029411764705882, m6 = 0.029411764705882,
                                 m7 = 0.117647058823529;
                    const double m8 = -0.083333333333333, m9 = 0.166666666666667, m10 = -0.166666666666667,
                                 m11 = 0.083333333333334;
                    const std::vector<double> f = slot_to_host(r, 1);
                    std::vector<double> energyR((size_t)r.n_p * rtb, 0.0);
                    for (int i = 0; i < r.n_x; i++)
                        for (int j = 0; j < r.n_p; j++) {
                            if (!r.nested.empty() && r.nested[r.ns(i, j)]) continue;
                            double f1 = f[pidx(i, j - 2, pit)], f2 = f[pidx(i, j - 1, pit)], f3 = f[pidx(i, j, pit)],
                                   f4 = f[pidx(i, j + 1, pit)], f5 = f[pidx(i, j + 2, pit)];
                            f5 -= f3;
                            f4 -= f3;
                            f2 -= f3;
                            f1 -= f3;
                            const double a1 = m0 * f1 + m1 * f2 + m2 * f4 + m3 * f5;
                            const double a2 = m4 * f1 + m5 * f2 + m6 * f4 + m7 * f5;
                            const double a3 = m8 * f1 + m9 * f2 + m10 * f4 + m11 * f5;
                            for (int k = 0; k < rtb; k++)
                                energyR[(size_t)j * rtb + k] += w[3 * k] * a1 + w[3 * k + 1] * a2 + w[3 * k + 2] * a3 + f3;
                        }
                    const double dx = s.GetDx(r.depth);
                    for (int k = 0; k < rtb; k++)
                        for (int j = 0; j < r.n_p; j++) energyR[(size_t)j * rtb + k] *= dx;
                    const size_t shift = (size_t)r.p_pos * rtb;  // Level::CollectEnergy
                    for (size_t q = 0; q < energyR.size(); q++) energyL[shift + q] += energyR[q];
                }
                for (size_t q = 0; q < energy.size(); q++) energy[q] += energyL[q];
            }
            std::ostringstream name;
            name << d << "/dNdP_" << sp << ".txt";
            line(out_stream(name.str(), digits), energy.data(), energy.size());
        }
    }
    if (mask & VX_OUT_POTENTIAL) {  // potential.txt (EMSolver.cpp:417-430)
        auto phi = to_host(F.phi, (size_t)n, eng->stream);
        line(out_stream(d + "/potential.txt", digits), phi.data(), phi.size());
    }
    if (mask & VX_OUT_EFIELD_LONG) {  // EFieldLong.txt: GetEfield(i) (EMSolver.cpp:381-394)
        auto ex = to_host(F.efin, (size_t)n, eng->stream);
        line(out_stream(d + "/EFieldLong.txt", digits), ex.data(), ex.size());
    }
    if (mask & VX_OUT_EFIELD_TRANS) {  // EFieldTrans.txt: E_y then E_z (EMSolver.cpp:396-415)
        std::ofstream &o = out_stream(d + "/EFieldTrans.txt", digits);
        auto ey = to_host(F.Ey, (size_t)nf, eng->stream), ez = to_host(F.Ez, (size_t)nf, eng->stream);
        line(o, ey.data(), ey.size());
        line(o, ez.data(), ez.size());
    }
    if (mask & VX_OUT_BFIELD_TRANS) {  // BFieldTrans.txt: B_y then B_z (EMSolver.cpp:432-451)
        std::ofstream &o = out_stream(d + "/BFieldTrans.txt", digits);
        auto by = to_host(F.By, (size_t)nf, eng->stream), bz = to_host(F.Bz, (size_t)nf, eng->stream);
        line(o, by.data(), by.size());
        line(o, bz.data(), bz.size());
    }
    if (mask & VX_OUT_ASQUARED) {  // ASquared.txt: GetASquared(i), i < x_size (EMSolver.cpp:453-466)
        auto a = to_host(F.asq, (size_t)n, eng->stream);
        line(out_stream(d + "/ASquared.txt", digits), a.data(), a.size());
    }
    if (mask & VX_OUT_TIME) {  // time.txt: the caller's clock (EMSolver.cpp:468-477)
        out_stream(d + "/time.txt", digits) << t << std::endl;
    }
}

// Mesh::outputRectangleData (Mesh.cpp:877-902): one file per species and non-empty level,
// every patch as "r x_pos p_pos n_x n_p" and then "x p  f" per cell (f of slot 0, four
// significant digits).
void Run::write_rectangles(const std::string &dir, double t) {
    eng->sync();
    const std::string d = dir.empty() ? std::string(".") : dir;
    for (size_t sp = 0; sp < rects.size(); sp++)
        for (size_t l = 0; l < rects[sp].size(); l++) {
            if (rects[sp][l].empty()) continue;
            std::ostringstream name;
            name << d << "/rectangleData_p" << sp << "_l" << l << "_t" << std::scientific << t << ".txt";
            std::ofstream o(name.str());
            if (!o) throw std::runtime_error("cannot open " + name.str());
            o << std::setprecision(4);
            for (auto &rp : rects[sp][l]) {
                const Rect &r = *rp;
                o << "r " << r.x_pos << " " << r.p_pos << " " << r.n_x << " " << r.n_p << "\n";
                const std::vector<double> f = slot_to_host(r, 0);
                for (int i = 0; i < r.n_x; i++)
                    for (int j = 0; j < r.n_p; j++)
                        o << r.x_pos + i << " " << r.p_pos + j << " " << std::scientific << " " << f[pidx(i, j, r.pitch)]
                          << "\n";
            }
        }
}

}  // namespace vx
