// Binary state exchange ("VXST0001") in the field / patch layout of the reference:
// fields as EMFieldSolver stores them (8 RK slots per array, EMSolver.cpp:20-26) and
// each patch's f as the reference's interleaved 3-slot block (Index3, Rectangle.hpp:96).
#include <cstdio>
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
    cudaStream_t st = eng.stream;
    auto put = [&](double *d, size_t expect) {
        auto v = f.rv();
        if (v.size() != expect) throw std::invalid_argument("state file array size mismatch");
        h2d(d, v, st);
        eng.sync();
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
                    h2d(dst, plane, st);
                    eng.sync();
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
    eng.refresh_efield(*this);
    eng.sync();
}

void Run::save_state(const std::string &path) {
    eng.sync();
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
    cudaStream_t st = eng.stream;
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
                    auto plane = d2h(src, r.plane_elems(), st);
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
