// Binary state exchange ("VXST0001") in the field / patch layout of the reference:
// fields as EMFieldSolver stores them (8 RK slots per array, EMSolver.cpp:20-26) and
// each patch's f as the reference's interleaved 3-slot block (Index3, Rectangle.hpp:96).
#include <cstdio>
#include <cmath>
#include <cstring>

#include "engine.hpp"

namespace vx {

namespace {
struct File {
    FILE *fp;
    File(const std::string &p, const char *mode) : fp(fopen(p.c_str(), mode)) {
        if (!fp) throw std::runtime_error("cannot open " + p);
    }
    ~File() {
        if (fp) fclose(fp);
    }
    void rd(void *p, size_t n) {
        if (n && fread(p, 1, n, fp) != n) throw std::runtime_error("truncated state file");
    }
    void wr(const void *p, size_t n) {
        if (n && fwrite(p, 1, n, fp) != n) throw std::runtime_error("write failed");
    }
    long long ri() {
        long long v;
        rd(&v, 8);
        return v;
    }
    double rdd() {
        double v;
        rd(&v, 8);
        return v;
    }
    std::vector<double> rv() {
        long long n = ri();
        if (n < 0 || n > (1ll << 36)) throw std::runtime_error("bad array length in state file");
        std::vector<double> v((size_t)n);
        rd(v.data(), v.size() * 8);
        return v;
    }
    void wi(long long v) { wr(&v, 8); }
    void wd(double v) { wr(&v, 8); }
    void wv(const std::vector<double> &v) {
        wi((long long)v.size());
        wr(v.data(), v.size() * 8);
    }
};

std::vector<double> d2h(const double *d, size_t n, cudaStream_t s) {
    std::vector<double> h(n);
    VX_CUDA(cudaMemcpyAsync(h.data(), d, n * 8, cudaMemcpyDeviceToHost, s));
    VX_CUDA(cudaStreamSynchronize(s));
    return h;
}
void h2d(double *d, const std::vector<double> &h, cudaStream_t s) {
    VX_CUDA(cudaMemcpyAsync(d, h.data(), h.size() * 8, cudaMemcpyHostToDevice, s));
}
// A patch plane in SI units: FP64 planes as they are, FP32 planes (scaled by fnorm)
// converted back.
std::vector<double> plane_to_host(const Rect &r, const double *d, double fnorm, cudaStream_t s) {
    if (r.esize == 8) return d2h(d, r.plane_elems(), s);
    std::vector<float> h(r.plane_elems());
    VX_CUDA(cudaMemcpyAsync(h.data(), d, r.plane_bytes(), cudaMemcpyDeviceToHost, s));
    VX_CUDA(cudaStreamSynchronize(s));
    std::vector<double> out(h.size());
    for (size_t q = 0; q < h.size(); q++) out[q] = (double)h[q] / fnorm;
    return out;
}
void plane_to_device(const Rect &r, double *d, const std::vector<double> &h, double fnorm, cudaStream_t s) {
    if (r.esize == 8) {
        h2d(d, h, s);
        VX_CUDA(cudaStreamSynchronize(s));
        return;
    }
    std::vector<float> h32(h.size());
    for (size_t q = 0; q < h.size(); q++) h32[q] = (float)(h[q] * fnorm);
    VX_CUDA(cudaMemcpyAsync(d, h32.data(), r.plane_bytes(), cudaMemcpyHostToDevice, s));
    VX_CUDA(cudaStreamSynchronize(s));
}
}  // namespace

void Run::load_state(const std::string &path) {
    File f(path, "rb");
    char magic[8];
    f.rd(magic, 8);
    if (std::memcmp(magic, "VXST0001", 8) != 0) throw std::runtime_error("not a VXST0001 state file");
    f.ri();  // step
    S->time = f.rdd();
    f.rdd();  // dt of the last step
    double ex0 = f.rdd();
    long long fn = f.ri(), fpre = f.ri(), fpost = f.ri();
    if (fn != n || fpre != pre || fpost != post) throw std::invalid_argument("state file grid does not match the run");
    cudaStream_t st = eng->stream;
    auto put = [&](double *d, size_t expect) {
        auto v = f.rv();
        if (v.size() != expect) throw std::invalid_argument("state file array size mismatch");
        h2d(d, v, st);
        eng->sync();
    };
    size_t fb = (size_t)nf * 8;
    put(F.By, fb);
    put(F.Bz, fb);
    put(F.Ey, fb);
    put(F.Ez, fb);
    put(F.Ay, fb);
    put(F.Az, fb);
    put(F.asq, (size_t)n + 1);
    put(F.phi, (size_t)n);
    put(F.charge, (size_t)n);
    put(F.J, (size_t)n);
    put(F.neut, (size_t)n);
    VX_CUDA(cudaMemcpyAsync(F.ex0, &ex0, 8, cudaMemcpyHostToDevice, st));
    long long ns = f.ri();
    if (ns != (long long)rects.size()) throw std::invalid_argument("state file species count mismatch");
    std::vector<std::vector<std::vector<std::unique_ptr<Rect>>>> nr(ns);
    std::vector<std::vector<double>> f1_host;  // FP32 runs: the loaded FP64 slot-1 planes
    bool fp32_exact = true;                     // every loaded f is an FP32-form value
    for (long long sp = 0; sp < ns; sp++) {
        long long nl = f.ri();
        if (nl != S->maxDepth + 1) throw std::invalid_argument("state file level count mismatch");
        nr[sp].resize(nl);
        for (long long l = 0; l < nl; l++) {
            long long nrect = f.ri();
            for (long long k = 0; k < nrect; k++) {
                auto r = std::make_unique<Rect>();
                r->x_pos = (int)f.ri();
                r->p_pos = (int)f.ri();
                r->n_x = (int)f.ri();
                r->n_p = (int)f.ri();
                r->depth = (int)f.ri();
                r->up = f.ri() != 0;
                r->down = f.ri() != 0;
                r->left = f.ri() != 0;
                r->right = f.ri() != 0;
                r->species = (int)sp;
                if (r->depth != l) throw std::invalid_argument("state file patch depth mismatch");
                auto fv = f.rv();
                size_t cells = (size_t)(r->n_x + 4) * (r->n_p + 4);
                if (fv.size() != 3 * cells) throw std::invalid_argument("state file patch size mismatch");
                allocate_rect(*r);
                for (int slot = 0; slot < 3; slot++) {
                    std::vector<double> plane(r->plane_elems(), 0.0);
                    for (int i = -2; i < r->n_x + 2; i++)
                        for (int j = -2; j < r->n_p + 2; j++)
                            plane[pidx(i, j, r->pitch)] = fv[3 * ((size_t)(r->n_p + 4) * (i + 2) + 2 + j) + slot];
                    double *dst = slot == 0 ? r->desc.f0 : (slot == 1 ? r->desc.f1 : r->desc.f2);
                    plane_to_device(*r, dst, plane, fnorm[sp], st);
                    if (slot == 1 && precision == kF32) {
                        const double fn = fnorm[sp];
                        for (double v : plane)
                            if ((double)(float)(v * fn) / fn != v) {
                                fp32_exact = false;
                                break;
                            }
                        f1_host.push_back(plane);
                    }
                }
                nr[sp][l].push_back(std::move(r));
            }
        }
    }
    rects = std::move(nr);
    build_amr();
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &rp : lvl) upload_rect_desc(*rp, 0);
    layout_version++;
    // a state written by an FP32 run holds FP32-form values already: nothing to rebase
    if (precision == kF32 && !fp32_exact) rebase_neutralization(f1_host);
    eng->refresh_efield(*this);
    eng->sync();
}

// The FP32 form represents f rounded to FP32, whose charge density differs from the
// FP64 state's by the rounding; the net charge of a plasma near neutrality is a small
// difference of large numbers, so that offset would show up as a spurious E_x.  After
// loading an FP64 state (one whose f values are not all FP32-form values), the
// neutralising background is shifted by
// (FP64 charge of the loaded f) - (FP32 charge of the rounded f), which makes the net
// charge of the loaded state the same in both forms.  The FP64 charge follows the
// column sums of Rectangle::CalculateRhoAndJ (Rectangle.cpp:157-282) and the level
// assembly (Level.cpp:19-62, EMSolver.cpp:104-122) on the host.
void Run::rebase_neutralization(const std::vector<std::vector<double>> &f1) {
    const Settings &s = *S;
    std::vector<std::vector<double>> colq(flat.size());
    for (size_t k = 0; k < flat.size(); k++) {
        const Rect &R = *flat[k];
        const int rtb = (int)std::pow(s.refinementRatio, R.depth);
        const double *f = f1[k].data();
        std::vector<double> w(3 * rtb);
        for (int i = 0; i < rtb; i++) {  // Rectangle.cpp:103-110
            double tl = -0.5 + i / (double)rtb, tr = -0.5 + (i + 1.0) / (double)rtb;
            w[3 * i] = (tl + tr) * 0.5;
            w[3 * i + 1] = (tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12);
            w[3 * i + 2] = (tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25;
        }
        auto rel = [&](int i, int j, int kk) {
            const double f3 = f[pidx(i, j, R.pitch)];
            if (rtb == 1) return f3;
            double g1 = f[pidx(i - 2, j, R.pitch)] - f3, g2 = f[pidx(i - 1, j, R.pitch)] - f3;
            double g4 = f[pidx(i + 1, j, R.pitch)] - f3, g5 = f[pidx(i + 2, j, R.pitch)] - f3;
            double a1 = 0.104166666666667 * g1 + -0.708333333333334 * g2 + 0.708333333333334 * g4 + -0.104166666666667 * g5;
            double a2 = 0.117647058823529 * g1 + 0.029411764705882 * g2 + 0.029411764705882 * g4 + 0.117647058823529 * g5;
            double a3 = -0.083333333333333 * g1 + 0.166666666666667 * g2 + -0.166666666666667 * g4 + 0.083333333333334 * g5;
            double te = 0.0, mine = 0.0;
            for (int q = 0; q < rtb; q++) {
                double v = w[3 * q] * a1 + w[3 * q + 1] * a2 + w[3 * q + 2] * a3 + f3;
                te += v;
                if (q == kk) mine = v;
            }
            return mine + (f3 - (1.0 / (double)rtb) * te);
        };
        const double dpq = s.GetDp(R.depth, R.species) * s.GetCharge(R.species);
        colq[k].assign((size_t)R.n_x * rtb, 0.0);
        for (int i = 0; i < R.n_x; i++)
            for (int kk = 0; kk < rtb; kk++) {
                double ch = 0.0;
                for (int j = 0; j < R.n_p; j++)
                    if (!R.nested[R.ns(i, j)]) ch += rel(i, j, kk);
                colq[k][(size_t)i * rtb + kk] = ch * dpq;
            }
    }
    std::vector<double> q64(n, 0.0);
    for (int x = 0; x < n; x++) {
        double charge = 0.0;
        for (auto &sp : rects) {
            double cs = 0.0;
            for (auto &lvl : sp) {
                double lc = 0.0;
                for (auto &rp : lvl) {
                    const Rect &R = *rp;
                    const int rtb = (int)std::pow(s.refinementRatio, R.depth);
                    int c = x - R.x_pos * rtb;
                    if (c >= 0 && c < R.n_x * rtb) lc += colq[R.id][c];
                }
                cs += lc;
            }
            charge += cs;
        }
        q64[x] = charge;
    }
    cudaStream_t st = eng->stream;
    auto keep_charge = d2h(F.charge, (size_t)n, st);
    auto keep_J = d2h(F.J, (size_t)n, st);
    auto neut = d2h(F.neut, (size_t)n, st);
    eng->moments_only({this});
    auto q32 = d2h(F.charge, (size_t)n, st);
    for (int x = 0; x < n; x++) neut[x] += q64[x] - q32[x];
    h2d(F.neut, neut, st);
    h2d(F.charge, keep_charge, st);
    h2d(F.J, keep_J, st);
    eng->sync();
}

void Run::save_state(const std::string &path) {
    eng->sync();
    File f(path, "wb");
    f.wr("VXST0001", 8);
    f.wi(0);
    f.wd(S->time);
    f.wd(0.0);
    double ex0;
    VX_CUDA(cudaMemcpy(&ex0, F.ex0, 8, cudaMemcpyDeviceToHost));
    f.wd(ex0);
    f.wi(n);
    f.wi(pre);
    f.wi(post);
    cudaStream_t st = eng->stream;
    size_t fb = (size_t)nf * 8;
    f.wv(d2h(F.By, fb, st));
    f.wv(d2h(F.Bz, fb, st));
    f.wv(d2h(F.Ey, fb, st));
    f.wv(d2h(F.Ez, fb, st));
    f.wv(d2h(F.Ay, fb, st));
    f.wv(d2h(F.Az, fb, st));
    f.wv(d2h(F.asq, (size_t)n + 1, st));
    f.wv(d2h(F.phi, (size_t)n, st));
    f.wv(d2h(F.charge, (size_t)n, st));
    f.wv(d2h(F.J, (size_t)n, st));
    f.wv(d2h(F.neut, (size_t)n, st));
    f.wi((long long)rects.size());
    for (auto &sp : rects) {
        f.wi((long long)sp.size());
        for (auto &lvl : sp) {
            f.wi((long long)lvl.size());
            for (auto &rp : lvl) {
                Rect &r = *rp;
                f.wi(r.x_pos);
                f.wi(r.p_pos);
                f.wi(r.n_x);
                f.wi(r.n_p);
                f.wi(r.depth);
                f.wi(r.up);
                f.wi(r.down);
                f.wi(r.left);
                f.wi(r.right);
                size_t cells = (size_t)(r.n_x + 4) * (r.n_p + 4);
                std::vector<double> fv(3 * cells, 0.0);
                for (int slot = 0; slot < 3; slot++) {
                    const double *src = slot == 0 ? r.desc.f0 : (slot == 1 ? r.desc.f1 : r.desc.f2);
                    auto plane = plane_to_host(r, src, fnorm[r.species], st);
                    for (int i = -2; i < r.n_x + 2; i++)
                        for (int j = -2; j < r.n_p + 2; j++)
                            fv[3 * ((size_t)(r.n_p + 4) * (i + 2) + 2 + j) + slot] = plane[pidx(i, j, r.pitch)];
                }
                f.wv(fv);
            }
        }
    }
}

}  // namespace vx
