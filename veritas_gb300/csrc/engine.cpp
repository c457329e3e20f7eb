#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "engine.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>

namespace vx {

bool g_launch_pdl = true;

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

DevBuf::DevBuf(size_t b) : bytes(b) {
    if (b) {
        VX_CUDA(cudaMalloc(&p, b));
        // Zero-fill and wait for it: later uploads run on a non-blocking stream that is
        // not ordered after the legacy default stream.  Only the legacy stream is waited
        // for, so a run built on one thread does not wait for steps running on another.
        VX_CUDA(cudaMemsetAsync(p, 0, b, cudaStreamLegacy));
        VX_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    }
}
DevBuf::DevBuf(size_t b, Uninit) : bytes(b) {
    if (b) VX_CUDA(cudaMalloc(&p, b));
}
DevBuf::~DevBuf() {
    if (p && own) cudaFree(p);
}
DevBuf &DevBuf::operator=(DevBuf &&o) noexcept {
    if (this != &o) {
        if (p && own) cudaFree(p);
        p = o.p;
        bytes = o.bytes;
        own = o.own;
        o.p = nullptr;
        o.bytes = 0;
    }
    return *this;
}

void TablePack::place(const DevBuf &arena) {
    if (arena.bytes < bytes()) throw std::logic_error("table storage smaller than its tables");
    base_ = arena.as<char>();
    for (const Item &it : items_)
        *it.view = DevBuf::view(base_ + (it.staged ? it.off : host_.size() + it.off), it.bytes);
}

void TablePack::copy(cudaStream_t s, void *pinned_host, void *pinned_dev) {
    if (host_.empty()) return;
    if (pinned_host && pinned_dev) {
        std::memcpy(pinned_host, host_.data(), host_.size());
        copy_from_host(pinned_dev, base_, host_.size(), s);  // host_.size() is a multiple of 256
    } else {
        VX_CUDA(cudaMemcpyAsync(base_, host_.data(), host_.size(), cudaMemcpyHostToDevice, s));
    }
}

// ---------------------------------------------------------------- Run
static_assert(sizeof(PatchT<float>) == sizeof(PatchT<double>), "descriptor layouts must match");

Run::Run(Engine &e, std::shared_ptr<Problem> prob, int prec) : eng(&e), precision(prec) {
    if (prec != kF64 && prec != kF32) throw std::invalid_argument("precision must be 64 or 32");
    Input grid;
    Particles particles;
    Output output;
    prob->initialConditions(grid, particles, output);
    S.reset(new Settings(grid, particles, output, prob));
    rects.resize(S->q.size());
    for (auto &sp : rects) sp.resize(S->maxDepth + 1);
    // the FP32 form stores f / (peak of the initial distribution)
    fnorm.assign(S->q.size(), 1.0);
    if (precision == kF32)
        for (size_t sp = 0; sp < fnorm.size(); sp++)
            if (S->fMax[sp] > 0) fnorm[sp] = 1.0 / S->fMax[sp];
    // Rectangle.cpp:94-101: weights onto the r sub-cells of a coarse cell
    const int r = S->refinementRatio;
    std::vector<double> w;
    for (int i = 0; i < r; i++) {
        double tl = -0.5 + i / (double)r;
        double tr = -0.5 + (i + 1.0) / (double)r;
        w.push_back((tl + tr) * 0.5);
        w.push_back((tl * tl + tl * tr + tr * tr) / 3.0 - (1.0 / 12));
        w.push_back((tl * tl * tl + tl * tl * tr + tl * tr * tr + tr * tr * tr) * 0.25);
    }
    drefc = DevBuf(w.size() * sizeof(double));
    VX_CUDA(cudaMemcpy(drefc.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice));
}

Run::~Run() {
    auto &v = eng->runs;
    v.erase(std::remove(v.begin(), v.end(), this), v.end());
    eng->forget(this);
}

void Run::migrate(Engine &to) {
    if (to.device != eng->device) throw std::invalid_argument("a run moves only between engines of one device");
    eng->forget(this);
    auto &v = eng->runs;
    v.erase(std::remove(v.begin(), v.end(), this), v.end());
    eng = &to;
}

long long Run::cell_count() const {
    long long c = 0;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) c += (long long)r->n_x * r->n_p;
    return c;
}

static const int kPlanes = 28;

void Run::allocate_rect(Rect &r) {
    r.pitch = ((r.n_p + 4) + 7) / 8 * 8;
    size_t pe = r.plane_elems();
    r.esize = precision == kF32 ? 4 : 8;
    // the FP32 form forms gamma and the face values in registers (fused face + flux
    // kernels): its patches have no planes for them
    const bool faces = precision != kF32;
    r.slab = DevBuf(pe * (faces ? kPlanes : kPlanes - 5) * r.esize);
    const int rtb = (int)std::pow(S->refinementRatio, r.depth);
    r.cols = DevBuf((size_t)2 * r.n_x * rtb * sizeof(double) + 64);
    PatchT<double> &d = r.desc;
    std::memset(&d, 0, sizeof d);
    char *base = r.slab.as<char>();
    int k = 0;
    auto plane = [&]() { return (double *)(base + pe * r.esize * (k++)); };
    d.f0 = plane();
    d.f1 = plane();
    d.f2 = plane();
    if (faces) {
        d.gam = plane();
        d.ex = plane();
        d.fx = plane();
        d.ep = plane();
        d.fp = plane();
    }
    for (int s = 0; s < 6; s++) d.FxH[s] = plane();
    for (int s = 0; s < 6; s++) d.FpH[s] = plane();
    d.FxL = plane();
    d.FpL = plane();
    d.FxDS = plane();
    d.FpDS = plane();
    d.Rp = plane();
    d.Rm = plane();
    d.Cx = plane();
    d.Cp = plane();
}

// Fill the geometric / physical part of a patch descriptor (Rectangle.cpp:7-113).
void Run::upload_rect_desc(Rect &r, int run_index) {
    const Settings &s = *S;
    PatchT<double> &d = r.desc;
    int sp = r.species;
    d.nx = r.n_x;
    d.np = r.n_p;
    d.x_pos = r.x_pos;
    d.p_pos = r.p_pos;
    d.depth = r.depth;
    d.rtb = (int)std::pow(s.refinementRatio, r.depth);
    d.pitch = r.pitch;
    d.xm = r.left ? 1 : 0;
    d.xp = r.right ? r.n_x : (r.n_x + 1);
    d.pp = r.up ? r.n_p : (r.n_p + 1);
    d.pm = r.down ? 1 : 0;
    d.run = run_index;
    d.species = sp;
    d.dp = s.GetDp(r.depth, sp);
    d.dx = s.GetDx(r.depth);
    d.dx_inv = 1 / d.dx;
    d.dp_inv = 1 / d.dp;
    d.pmin = s.pmin[sp];
    d.q = s.GetCharge(sp);
    d.qq = d.q * d.q;
    d.mass = s.GetMass(sp);
    d.cc = kCs * kCs * s.GetMass(sp);
    double m_inv = 1 / s.GetMass(sp);
    d.g2 = (m_inv * kCInv) * (m_inv * kCInv);
    d.fnorm = fnorm[sp];
    d.pnorm = m_inv * kCInv;
    d.dpn = d.dp * d.pnorm;
    d.kx = d.dp_inv * d.cc;
    d.kp = d.cc * d.dx_inv;
    d.weno_eps = (float)std::max(1e-10 * d.fnorm * d.fnorm, 1e-30);
    d.pminf = (float)(d.pmin * d.pnorm);
    d.dpnf = (float)d.dpn;
    d.kxf = (float)d.kx;
    d.kpf = (float)d.kp;
    d.dxif = (float)d.dx_inv;
    d.dpif = (float)d.dp_inv;
    d.qf = (float)d.q;
    d.a2nf = (float)(d.qq * d.g2);
    d.msc_rho = (1.0 / d.fnorm) * (d.dp * d.q);
    d.msc_j = (1.0 / d.fnorm) * (1.0 / ((1.0 / d.mass) * kCInv)) * (-d.q * d.q / d.mass);
    if (precision == kF32 && d.rtb != 1 && d.rtb != 2 && d.rtb != 4 && d.rtb != 8)
        throw std::invalid_argument("the FP32 form supports 1, 2, 4 or 8 finest cells per coarse cell");
    double *cols = r.cols.as<double>();
    d.chargeR = cols;
    d.currentR = cols + (size_t)r.n_x * d.rtb;
    d.r = (int)s.refinementRatio;
    d.relc = drelc.p ? drelc.as<double>() + relc_off[r.depth] : nullptr;
    d.refc = drefc.as<double>();
    d.relc32 = drelc32.p ? drelc32.as<float>() + relc32_off[r.depth] : nullptr;
    if (r.masks.p) {
        const size_t pe = r.plane_elems();
        uint8_t *m = r.masks.as<uint8_t>();
        d.nested = m;
        d.ifx = m + pe;
        d.ifp = m + 2 * pe;
        d.has_iface = 1;
    } else {
        d.nested = d.ifx = d.ifp = nullptr;
        d.has_iface = 0;
    }
}

// Rectangle::InitializeDistribution, non-MKL quadrature (Rectangle.cpp:616-665), run on
// host threads with the user's InitialDistribution hook.
void Run::init_rect_distribution(Rect &r) {
    const Settings &s = *S;
    const int nvals = std::pow(s.refinementRatio, r.depth + s.quadratureDepth);
    const double dx = s.GetDx(r.depth), dp = s.GetDp(r.depth, r.species);
    const double pmin = s.pmin[r.species];
    if (precision == kF32 && s.problem->Separable()) {
        // same sample points, summed as (sum_k density)(sum_l profile)
        std::vector<double> dx_sum(r.n_x, 0.0), dp_sum(r.n_p, 0.0);
        for (int i = 0; i < r.n_x; i++)
            for (int k = 0; k < nvals; k++) dx_sum[i] += s.problem->Density(s, ((0.5 + k) / nvals + i + r.x_pos) * dx, r.species);
        for (int j = 0; j < r.n_p; j++)
            for (int l = 0; l < nvals; l++)
                dp_sum[j] += s.problem->Profile(s, pmin + dp * ((0.5 + l) / nvals + j + r.p_pos), r.species);
        // the product on the device (the planes of a new patch are zero: ghosts stay 0)
        const double inv = 1 / std::pow(nvals, 2.0);
        DevBuf dxs = upload(dx_sum, eng->stream), dps = upload(dp_sum, eng->stream);
        launch_fill_separable((float *)r.desc.f0, (float *)r.desc.f1, r.pitch, r.n_x, r.n_p, dxs.as<double>(),
                              dps.as<double>(), inv, fnorm[r.species], eng->stream);
        VX_CUDA(cudaStreamSynchronize(eng->stream));
        return;
    }
    const int terms = precision == kF64 ? s.problem->ProductTerms(r.species) : 0;
    if (terms > 0) {
        // the hook's factors at every sample point on the host, the double sum on the device
        std::vector<double> X((size_t)terms * r.n_x * nvals), Pf((size_t)terms * r.n_p * nvals), C(terms);
        for (int t = 0; t < terms; t++) {
            C[t] = s.problem->Divisor(s, t, r.species);
            for (int i = 0; i < r.n_x; i++)
                for (int k = 0; k < nvals; k++)
                    X[((size_t)t * r.n_x + i) * nvals + k] =
                        s.problem->XFactor(s, t, ((0.5 + k) / nvals + i + r.x_pos) * dx, r.species);
            for (int j = 0; j < r.n_p; j++)
                for (int l = 0; l < nvals; l++)
                    Pf[((size_t)t * r.n_p + j) * nvals + l] =
                        s.problem->PFactor(s, t, pmin + dp * ((0.5 + l) / nvals + j + r.p_pos), r.species);
        }
        DevBuf dX = upload(X, eng->stream), dP = upload(Pf, eng->stream), dC = upload(C, eng->stream);
        launch_quadrature64((double *)r.desc.f0, (double *)r.desc.f1, r.pitch, r.n_x, r.n_p, nvals, terms,
                            dX.as<double>(), dP.as<double>(), dC.as<double>(), 1 / std::pow(nvals, 2.0), eng->stream);
        VX_CUDA(cudaStreamSynchronize(eng->stream));
        return;
    }
    std::vector<double> host((size_t)(r.n_x + 4) * r.pitch, 0.0);
    unsigned nth = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; t++) {
        th.emplace_back([&, t]() {
            for (int i = (int)t; i < r.n_x; i += (int)nth) {
                for (int j = 0; j < r.n_p; j++) {
                    double temp = 0.0, xp = 0.0, pp = 0.0;
                    for (int k = 0; k < nvals; k++) {
                        for (int l = 0; l < nvals; l++) {
                            xp = ((0.5 + k) / nvals + i + r.x_pos) * dx;
                            pp = pmin + dp * ((0.5 + l) / nvals + j + r.p_pos);
                            temp += s.InitialDistribution(xp, pp, r.species);
                        }
                    }
                    host[pidx(i, j, r.pitch)] = temp * (1 / std::pow(nvals, 2.0));
                }
            }
        });
    }
    for (auto &x : th) x.join();
    if (r.esize == 4) {
        std::vector<float> h32(host.size());
        const double fn = fnorm[r.species];
        for (size_t q = 0; q < host.size(); q++) h32[q] = (float)(host[q] * fn);
        VX_CUDA(cudaMemcpyAsync(r.desc.f0, h32.data(), r.plane_bytes(), cudaMemcpyHostToDevice, eng->stream));
        VX_CUDA(cudaMemcpyAsync(r.desc.f1, h32.data(), r.plane_bytes(), cudaMemcpyHostToDevice, eng->stream));
        VX_CUDA(cudaStreamSynchronize(eng->stream));
        return;
    }
    size_t bytes = host.size() * sizeof(double);
    VX_CUDA(cudaMemcpyAsync(r.desc.f0, host.data(), bytes, cudaMemcpyHostToDevice, eng->stream));
    VX_CUDA(cudaMemcpyAsync(r.desc.f1, host.data(), bytes, cudaMemcpyHostToDevice, eng->stream));
    VX_CUDA(cudaStreamSynchronize(eng->stream));
}

void Run::alloc_fields() {
    const Settings &s = *S;
    n = s.x_size_finest;
    pre = std::max(std::floor(s.preLength / s.GetDx(0)), 2.0);
    post = std::max(std::floor(s.postLength / s.GetDx(0)), 2.0);
    nf = n + pre + post;
    dx0 = s.GetDx(0);
    size_t fb = (size_t)nf * 8 * sizeof(double);
    dBy = DevBuf(fb);
    dBz = DevBuf(fb);
    dEy = DevBuf(fb);
    dEz = DevBuf(fb);
    dAy = DevBuf(fb);
    dAz = DevBuf(fb);
    dasq = DevBuf((size_t)(n + 1) * sizeof(double));
    dphi = DevBuf((size_t)n * sizeof(double));
    dcharge = DevBuf((size_t)n * sizeof(double));
    dJ = DevBuf((size_t)n * sizeof(double));
    dneut = DevBuf((size_t)n * sizeof(double));
    defin = DevBuf((size_t)n * sizeof(double));
    dex0 = DevBuf(sizeof(double));
    dasq32 = DevBuf((size_t)(n + 1) * sizeof(float));
    defin32 = DevBuf((size_t)n * sizeof(float));
    dacell32 = DevBuf((size_t)nf * sizeof(float));
    F.n = n;
    F.pre = pre;
    F.post = post;
    F.nf = nf;
    F.dx0 = dx0;
    F.By = dBy.as<double>();
    F.Bz = dBz.as<double>();
    F.Ey = dEy.as<double>();
    F.Ez = dEz.as<double>();
    F.Ay = dAy.as<double>();
    F.Az = dAz.as<double>();
    F.asq = dasq.as<double>();
    F.phi = dphi.as<double>();
    F.charge = dcharge.as<double>();
    F.J = dJ.as<double>();
    F.neut = dneut.as<double>();
    F.efin = defin.as<double>();
    F.ex0 = dex0.as<double>();
    F.acell32 = dacell32.as<float>();
    F.asq32 = dasq32.as<float>();
    F.efin32 = defin32.as<float>();
}

void Run::upload_lu() {
    cudaStream_t st = eng->stream;
    auto Lb = lu.lower_band();
    auto Ub = lu.upper_band();
    pipe_rfc = lu.first_read_chunk(Lb, kPoisRowsHost);
    dlu_perm = upload(lu.perm, st);
    dlb_band = upload(Lb.band, st);
    dlb_fptr = upload(Lb.fptr, st);
    dlb_fcol = upload(Lb.fcol, st);
    dlb_fval = upload(Lb.fval, st);
    dlb_slot = upload(Lb.slot_coef, st);
    dlb_sload = upload(Lb.slot_load, st);
    dlb_take = upload(Lb.take, st);
    dub_band = upload(Ub.band, st);
    dub_diag = upload(Ub.diag, st);
    dub_rdiag = upload(Ub.rdiag, st);
    dub_rdlo = upload(Ub.rdiag_lo, st);
    dub_fptr = upload(Ub.fptr, st);
    dub_fcol = upload(Ub.fcol, st);
    dub_fval = upload(Ub.fval, st);
    eng->sync();
    ludev.n = lu.n;
    ludev.perm = dlu_perm.as<int>();
    ludev.L = BandFactor{dlb_band.as<double>(), nullptr, nullptr, nullptr, dlb_fptr.as<int>(), dlb_fcol.as<int>(),
                         dlb_fval.as<double>(), Lb.nslots, dlb_slot.as<double>(), dlb_sload.as<int>(),
                         dlb_take.as<int>(), -1};
    ludev.U = BandFactor{dub_band.as<double>(), dub_diag.as<double>(), dub_rdiag.as<double>(), dub_rdlo.as<double>(),
                         dub_fptr.as<int>(),
                         dub_fcol.as<int>(), dub_fval.as<double>(), -1, nullptr, nullptr, nullptr, Ub.far_pre_col};
}

// SolverManager::SolverManager (SolverManager.cpp:8-26).  Mesh::Mesh (Mesh.cpp:8-50):
// the base level alone (the reference's initial flagging adds nothing here, its
// non-MKL branch collects no cells), then maxDepth rounds of ghost fill + regrid with
// every new patch set from the quadrature.  Then the field solver and neutralisation.
void Run::init() {
    const Settings &s = *S;
    // VX_TRACE_INIT=1: wall time of each phase on stderr (serving diagnostics)
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        eng->sync();
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "vx init %-14s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
    std::vector<std::vector<BoxList>> hier(rects.size());
    for (size_t sp = 0; sp < rects.size(); sp++)
        hier[sp] = {BoxList{{{0, 0}, {s.GetXSize(s.maxDepth), s.GetPSize(s.maxDepth, (int)sp)}}}};
    promote(hier, true);
    lap("base patch");
    for (int i = 0; i < s.maxDepth; i++) {
        push_data(1);
        regrid(true);
        lap("regrid round");
    }
    alloc_fields();
    push_data(1);
    lap("fields");
    if (precision == kF32) poisson = kPoissonScan;
    if (poisson == kPoissonScan) {
        build_poisson_fast();
    } else {
        int info = lu.build(n);
        if (info) throw std::runtime_error("Poisson operator is singular");
        upload_lu();
    }
    lap("poisson setup");
    layout_version++;
    enforce_neutralization();
    lap("neutralisation");
}

// EMFieldSolver::EnforceChargeNeutralization (EMSolver.cpp:621-629):
// neutralizationCharge = -rho(t=0), J = 0.
void Run::enforce_neutralization() {
    eng->moments_only({this});
    launch_negate(F.neut, F.charge, n, eng->stream);
    VX_CUDA(cudaMemsetAsync(F.J, 0, (size_t)n * sizeof(double), eng->stream));
    eng->sync();
}

int64_t Run::state_size() const {
    int64_t len = 0;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) len += (int64_t)((r->plane_bytes() + 7) / 8);
    return len + 6 * (int64_t)nf + (n + 1) + n + 1;
}

// Host-buffer step: H2D of the packed state, one RK step, D2H of the new state.
void Run::step_host(const double *in, double *out, double dt) {
    cudaStream_t st = eng->stream;
    const double *p = in;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) {
                // FP32 runs pack the scaled float plane two values per double slot
                size_t b = r->plane_bytes();
                VX_CUDA(cudaMemcpyAsync(r->desc.f0, p, b, cudaMemcpyHostToDevice, st));
                VX_CUDA(cudaMemcpyAsync(r->desc.f1, r->desc.f0, b, cudaMemcpyDeviceToDevice, st));
                p += (b + 7) / 8;
            }
    for (double *X : {F.By, F.Bz, F.Ey, F.Ez, F.Ay, F.Az}) {
        VX_CUDA(cudaMemcpyAsync(X, p, (size_t)nf * sizeof(double), cudaMemcpyHostToDevice, st));
        VX_CUDA(cudaMemcpyAsync(X + nf, X, (size_t)nf * sizeof(double), cudaMemcpyDeviceToDevice, st));
        p += nf;
    }
    VX_CUDA(cudaMemcpyAsync(F.asq, p, (size_t)(n + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
    p += n + 1;
    VX_CUDA(cudaMemcpyAsync(F.phi, p, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
    p += n;
    VX_CUDA(cudaMemcpyAsync(F.ex0, p, sizeof(double), cudaMemcpyHostToDevice, st));
    eng->refresh_efield(*this);
    advance(dt);
    state_to_host(out);
}

void Run::state_to_host(double *out) {
    cudaStream_t st = eng->stream;
    double *q = out;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) {
                VX_CUDA(cudaMemcpyAsync(q, r->desc.f0, r->plane_bytes(), cudaMemcpyDeviceToHost, st));
                q += (r->plane_bytes() + 7) / 8;
            }
    for (double *X : {F.By, F.Bz, F.Ey, F.Ez, F.Ay, F.Az}) {
        VX_CUDA(cudaMemcpyAsync(q, X, (size_t)nf * sizeof(double), cudaMemcpyDeviceToHost, st));
        q += nf;
    }
    VX_CUDA(cudaMemcpyAsync(q, F.asq, (size_t)(n + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
    q += n + 1;
    VX_CUDA(cudaMemcpyAsync(q, F.phi, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
    q += n;
    VX_CUDA(cudaMemcpyAsync(q, F.ex0, sizeof(double), cudaMemcpyDeviceToHost, st));
    eng->sync();
}

double Run::calculate_dt() { return eng->calculate_dt({this})[0]; }

void Run::advance(double dt) { eng->advance({this}, {dt}); }

void Run::advance_fields(double dt) { eng->advance_fields({this}, {dt}); }

// ---------------------------------------------------------------- LaunchSet / Engine
LaunchSet::~LaunchSet() {
    if (graph) cudaGraphExecDestroy(graph);
}

Engine::Engine(int dev) : device(dev) {
    VX_CUDA(cudaSetDevice(dev));
    VX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    VX_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    VX_CUDA(cudaEventCreateWithFlags(&ev_pinned_, cudaEventDisableTiming));
    VX_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    VX_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    VX_CUDA(cudaEventCreateWithFlags(&ev_gamma, cudaEventDisableTiming));
    VX_CUDA(cudaEventCreateWithFlags(&ev_mx, cudaEventDisableTiming));
    int lo = 0, hi = 0;
    VX_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    prio_hi_ = hi;
    VX_CUDA(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
}

Engine::~Engine() {
    sets_.clear();
    arena_cache_.clear();
    if (pinned_) cudaFreeHost(pinned_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_gamma) cudaEventDestroy(ev_gamma);
    if (ev_mx) cudaEventDestroy(ev_mx);
    if (ev_pinned_) cudaEventDestroy(ev_pinned_);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
}

void Engine::timer_begin() {
    if (!ev0_) {
        VX_CUDA(cudaEventCreate(&ev0_));
        VX_CUDA(cudaEventCreate(&ev1_));
    }
    VX_CUDA(cudaEventRecord(ev0_, stream));
}

double Engine::timer_end() {
    if (!ev0_) throw std::logic_error("timer_end without timer_begin");
    VX_CUDA(cudaEventRecord(ev1_, stream));
    VX_CUDA(cudaEventSynchronize(ev1_));
    float ms = 0;
    VX_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
    return ms;
}

void Engine::flush_l2() {
    if (!flush_.p) flush_ = DevBuf((size_t)512 << 20);
    VX_CUDA(cudaMemsetAsync(flush_.p, (int)(kernel_launches & 0xff), flush_.bytes, stream));
}

double Engine::measure_fp64_peak() {
    if (!flush_.p) flush_ = DevBuf((size_t)512 << 20);
    int sms = 0;
    VX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int iters = 4096;
    int blocks = sms * 8, threads = 256;
    launch_fp64_peak(flush_.as<double>(), blocks, threads, iters, stream);
    timer_begin();
    launch_fp64_peak(flush_.as<double>(), blocks, threads, iters, stream);
    double ms = timer_end();
    kernel_launches += 2;
    double flops = 2.0 * 8.0 * (double)iters * blocks * threads;  // 8 independent FMA chains
    return flops / (ms * 1e-3) / 1e9;
}

void Engine::measure_fp64_latency(double *mul_sub_cycles, double *shfl_cycles) {
    if (!flush_.p) flush_ = DevBuf((size_t)512 << 20);
    const int iters = 4096;
    long long *cyc = flush_.as<long long>();
    double *val = flush_.as<double>() + 2;
    launch_fp64_latency(cyc, val, iters, stream);  // warm-up
    launch_fp64_latency(cyc, val, iters, stream);
    kernel_launches += 2;
    long long h[2];
    VX_CUDA(cudaMemcpyAsync(h, cyc, sizeof h, cudaMemcpyDeviceToHost, stream));
    VX_CUDA(cudaStreamSynchronize(stream));
    *mul_sub_cycles = (double)h[0] / iters;
    *shfl_cycles = (double)(h[1] - h[0]) / iters;
}

// Precision dispatch of the per-stage kernels of a launch set.
static void fct_sub(const LaunchSet &L, const FctLaunch &fl, int sub) {
    if (L.precision == kF32) launch_fct32_substep(fl, sub);
    else if (L.fast64) launch_fct64_substep_fast(fl, sub);
    else launch_fct64_substep(fl, sub);
}
static void run_moments(const LaunchSet &L, const MomLaunch &ml) {
    if (L.precision == kF32) launch_moments32(ml);
    else launch_moments64(ml);
}
static void run_poisson(const LaunchSet &L, const PoissonLaunch &pl) {
    if (L.poisson == kPoissonScan) {
        PoissonFastLaunch f{};
        f.pf = L.dpf.as<PoissonFastDev>();
        f.fields = pl.fields;
        f.w = pl.w;
        f.fcoef = pl.fcoef;
        f.nruns = pl.nruns;
        f.maxn = pl.maxn;
        f.f32 = L.precision == kF32;
        f.stream = pl.stream;
        launch_poisson_fast(f);
    } else {
        launch_poisson(pl);
    }
}

std::vector<double> Engine::profile_kernels(Run &run, int reps) {
    LaunchSet &L = get_set({&run});
    FctLaunch fl{};
    fl.patches = L.dpatch.p;
    fl.tiles = L.dtiles.as<TileRef>();
    fl.ntiles = L.ntiles;
    fl.tile_j = L.tile_j;
    fl.tile_i = L.tile_i;
    fl.xtiles = L.dxtiles.as<TileRef>();
    fl.ptiles = L.dptiles.as<TileRef>();
    fl.nxtiles = L.nxtiles;
    fl.nptiles = L.nptiles;
    fl.fields = L.dfields.as<RunFields>();
    fl.params = L.dparams.as<double>();
    fl.params32 = L.dparams32.as<float>();
    fl.step = 0;
    fl.stream = stream;
    std::vector<double> out;
    auto time_it = [&](auto &&fn) {
        fn();
        timer_begin();
        for (int r = 0; r < reps; r++) fn();
        out.push_back(timer_end() / reps);
        kernel_launches += reps + 1;
    };
    // stage-0 parameters with dt = 0 keep every kernel well defined
    // FP32 sets run the fused face + flux kernels: "faces" and "flux" time the x and p
    // ones, "gamma" (folded into them) reads 0
    for (int sub : {kSubGamma, kSubFaces, kSubFlux, kSubDsF2, kSubLimR, kSubLimC, kSubUpdate}) {
        if (L.precision == kF32 && sub == kSubGamma) {
            out.push_back(0.0);
            continue;
        }
        const int run = L.precision == kF32 && sub == kSubFaces ? kSubXFlux
                        : L.precision == kF32 && sub == kSubFlux ? kSubPFlux
                                                                  : sub;
        time_it([&] { fct_sub(L, fl, run); });
    }
    MomLaunch ml{};
    ml.patches = L.dpatch.p;
    ml.colpatch = L.dcolpatch.as<int>();
    ml.colidx = L.dcolidx.as<int>();
    ml.ncols = L.ncols;
    ml.maxnp = L.maxnp;
    ml.fields = L.dfields.as<RunFields>();
    ml.nruns = (int)L.runs.size();
    ml.maxnf = L.maxnf;
    ml.fast = L.precision == kF64 ? L.fast64 : 0;
    ml.acell = 0;  // as in a step's later stages: the Maxwell stage made the copy
    ml.stream = stream;
    time_it([&] { run_moments(L, ml); });
    AsmLaunch al{};
    al.patches = L.dpatch.p;
    al.lvl_ptr = L.dlvl_ptr.as<int>();
    al.lvl_off = L.dlvl_off.as<int>();
    al.lvl_patch = L.dlvl_patch.as<int>();
    al.run_n = L.drun_n.as<int>();
    al.run_ns = L.drun_ns.as<int>();
    al.run_nl = L.drun_nl.as<int>();
    al.nruns = 1;
    al.maxn = L.maxn;
    al.pairs = L.precision == kF32 ? 1 : 0;
    al.fields = L.dfields.as<RunFields>();
    al.stream = stream;
    time_it([&] { launch_assemble(al); });
    PoissonLaunch pl{};
    pl.lu = L.dlu.as<LUDev>();
    pl.fields = L.dfields.as<RunFields>();
    pl.w = L.dw.as<double>();
    pl.fcoef = L.dfcoef.as<double>();
    pl.nruns = 1;
    pl.maxn = L.maxn;
    pl.stream = stream;
    time_it([&] { run_poisson(L, pl); });
    // VX_TRACE_POISSON=1 (LU solve): clock64 at each chunk end of both sweeps, on stderr
    if (std::getenv("VX_TRACE_POISSON") && L.poisson == kPoissonLU) {
        const int nch = (L.maxn + kPoisRowsHost - 1) / kPoisRowsHost;
        DevBuf tr((size_t)(2 * nch + 2) * sizeof(unsigned long long));
        pl.trace = tr.as<unsigned long long>();
        run_poisson(L, pl);
        sync();
        std::vector<unsigned long long> h(2 * nch + 1);
        VX_CUDA(cudaMemcpy(h.data(), tr.p, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        std::fprintf(stderr, "vx poisson n=%d chunks=%d forward %llu cycles, backward %llu cycles\n", L.maxn, nch,
                     h[nch] - h[0], h[2 * nch] - h[nch]);
        for (int c = 0; c < 2 * nch; c++) std::fprintf(stderr, "  chunk %d: %llu\n", c, h[c + 1] - h[c]);
        pl.trace = nullptr;
    }
    MaxwellLaunch mx{};
    mx.fields = L.dfields.as<RunFields>();
    mx.nruns = 1;
    mx.maxnf = L.maxnf;
    mx.params = L.dparams.as<double>();
    mx.dxinv = L.ddxinv.as<double>();
    mx.step = 0;
    mx.f32 = L.precision == kF32;
    mx.stream = stream;
    time_it([&] { launch_maxwell(mx); });
    // the AMR op batches of one stage (each entry: all batches of that kind)
    time_it([&] {
        for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++)
            launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 1, L.precision, stream);
    });
    time_it([&] {
        for (size_t b = 0; b + 1 < L.iface_ptr.size(); b++)
            launch_iface(L.dpatch.p, L.diface.as<IfaceOp>() + L.iface_ptr[b], L.iface_ptr[b + 1] - L.iface_ptr[b], 0, L.precision, stream);
    });
    time_it([&] {
        for (size_t b = 0; b + 1 < L.csync_ptr.size(); b++)
            launch_csync(L.dpatch.p, L.dcsync.as<CSyncOp>() + L.csync_ptr[b], L.csync_ptr[b + 1] - L.csync_ptr[b], L.precision, stream);
    });
    // FP64 exact-solve runs: the pipelined moments + assembly + solve launch (alone here,
    // without the face kernels that share the GPU with it inside a step)
    if (L.pipe) {
        StageLaunches K = stage_launches(L);
        K.ml.acell = 0;
        PipeLaunch P = pipe_launch(L, K);
        time_it([&] { launch_moments_poisson64(P); });
        pipe_pending_ = true;
        // VX_TRACE_PIPE=1: when each forward chunk's rows were ready, when the sweeps ended
        // and when each chunk's last moment unit finished (ns from the solve's start)
        if (std::getenv("VX_TRACE_PIPE")) {
            const int nch = (L.runs[0]->n + kPoisRowsHost - 1) / kPoisRowsHost;
            DevBuf tr((size_t)(3 + 2 * nch) * sizeof(unsigned long long));
            DevBuf tp((size_t)(2 * nch + 2) * sizeof(unsigned long long));
            P.trace = tr.as<unsigned long long>();
            P.trace_nch = nch;
            P.P.trace = tp.as<unsigned long long>();
            launch_moments_poisson64(P);
            sync();
            std::vector<unsigned long long> a(3 + 2 * nch), b(2 * nch + 1);
            VX_CUDA(cudaMemcpy(a.data(), tr.p, a.size() * sizeof(a[0]), cudaMemcpyDeviceToHost));
            VX_CUDA(cudaMemcpy(b.data(), tp.p, b.size() * sizeof(b[0]), cudaMemcpyDeviceToHost));
            const double t0 = (double)a[0];
            std::fprintf(stderr, "vx pipe n=%d chunks=%d units=%d (us from the solve's start)\n", L.runs[0]->n, nch,
                         L.pipe_nunits);
            std::fprintf(stderr, "  forward sweep: %llu cycles in %.1f us\n", a[2 + 2 * nch] - a[1 + 2 * nch],
                         (b[nch] - b[0]) * 1e-3);
            for (int c = 0; c < nch; c++)
                std::fprintf(stderr, "  chunk %2d: units done %8.1f rows ready %8.1f forward end %8.1f backward end %8.1f\n",
                             c, a[1 + nch + c] ? (a[1 + nch + c] - t0) * 1e-3 : -1.0, (a[1 + c] - t0) * 1e-3,
                             (b[1 + c] - t0) * 1e-3, (b[1 + nch + (nch - 1 - c)] - t0) * 1e-3);
        }
    } else {
        out.push_back(0.0);
    }
    return out;
}

void Engine::sync() {
    VX_CUDA(cudaStreamSynchronize(stream));
    check_device_errors();
}

DevBuf Engine::take_arena(size_t bytes) {
    // a cached block of at least `bytes` and at most twice that (plus 1 MiB)
    auto it = arena_cache_.lower_bound(bytes);
    if (it != arena_cache_.end() && it->first <= 2 * bytes + ((size_t)1 << 20)) {
        DevBuf b = std::move(it->second);
        arena_cache_bytes_ -= it->first;
        arena_cache_.erase(it);
        return b;
    }
    // new storage rounded up (1/8 and to 256 KiB) so that later sets of a similar mix fit
    const size_t cap = (bytes + bytes / 8 + ((size_t)256 << 10) - 1) / ((size_t)256 << 10) * ((size_t)256 << 10);
    return DevBuf(cap, DevBuf::Uninit{});
}

void *Engine::pinned_staging(size_t bytes) {
    if (bytes > pinned_bytes_) {
        if (pinned_) cudaFreeHost(pinned_);
        pinned_ = pinned_dev_ = nullptr;
        pinned_bytes_ = 0;
        const size_t cap = std::max(bytes + bytes / 2, (size_t)4 << 20);
        VX_CUDA(cudaHostAlloc(&pinned_, cap, cudaHostAllocMapped));
        VX_CUDA(cudaHostGetDevicePointer(&pinned_dev_, pinned_, 0));
        pinned_bytes_ = cap;
    }
    return pinned_;
}

void Engine::drop_idle(std::unique_ptr<LaunchSet> &L) {
    DevBuf a = std::move(L->arena);
    L.reset();
    if (!a.p || !a.own) return;
    if (a.bytes > arena_cache_limit) return;  // freed
    while (arena_cache_bytes_ + a.bytes > arena_cache_limit && !arena_cache_.empty()) {
        auto it = arena_cache_.begin();  // the smallest goes first
        arena_cache_bytes_ -= it->first;
        arena_cache_.erase(it);
    }
    arena_cache_bytes_ += a.bytes;
    const size_t cap = a.bytes;
    arena_cache_.emplace(cap, std::move(a));
}

// Drop every cached launch set that refers to a run being destroyed.
void Engine::forget(Run *r) {
    cudaStreamSynchronize(stream);
    for (auto it = sets_.begin(); it != sets_.end();) {
        if (std::find(it->first.begin(), it->first.end(), r) != it->first.end()) {
            drop_idle(it->second);
            it = sets_.erase(it);
        } else {
            ++it;
        }
    }
}

void Engine::set_launch_mode(bool graphs, bool pdl) {
    sync();
    use_graphs = graphs;
    g_launch_pdl = pdl;
    for (auto &kv : sets_)
        if (kv.second->graph) {
            cudaGraphExecDestroy(kv.second->graph);
            kv.second->graph = nullptr;
        }
}

void Engine::retain_sets(const std::vector<std::vector<Run *>> &keep) {
    bool drop = false;
    for (auto &kv : sets_)
        if (std::find(keep.begin(), keep.end(), kv.first) == keep.end()) drop = true;
    if (!drop) return;
    sync();  // a dropped set's buffers may still be in use by queued work
    for (auto it = sets_.begin(); it != sets_.end();) {
        if (std::find(keep.begin(), keep.end(), it->first) == keep.end()) {
            drop_idle(it->second);  // synchronised above
            it = sets_.erase(it);
        } else {
            ++it;
        }
    }
}

LaunchSet &Engine::get_set(const std::vector<Run *> &set, bool defer) {
    auto it = sets_.find(set);
    uint64_t ver = 0;
    for (Run *r : set) ver = ver * 1000003ull + r->layout_version;
    if (it != sets_.end() && it->second->key_version == ver) {
        if (!defer) flush_set(*it->second);
        return *it->second;
    }
    auto L = std::make_unique<LaunchSet>();
    L->runs = set;
    L->key_version = ver;
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    build_set(*L);
    if (!defer) flush_set(*L);
    if (trace) {
        std::fprintf(stderr, "vx launch set of %zu runs: %8.2f ms\n", set.size(),
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    LaunchSet &ref = *L;
    sets_[set] = std::move(L);
    return ref;
}

// Tile list covering every patch's padded block with tile_j (p) x tile_i (x) tiles.
void Engine::build_tiles(LaunchSet &L, TablePack *pk) {
    TablePack alone;
    TablePack &P = pk ? *pk : alone;
    // FP32 streaming kernels own four p cells per thread: 128-cell tiles starting at
    // j0 = -2 + 128 k keep every thread's cells one aligned float4
    if (L.precision == kF32) L.tile_j = 128;
    std::vector<TileRef> tiles;
    int pi = 0;
    for (Run *R : L.runs)
        for (auto &sp : R->rects)
            for (auto &lvl : sp)
                for (auto &rp : lvl) {
                    for (int i0 = -2; i0 <= rp->n_x + 1; i0 += L.tile_i)
                        for (int j0 = -2; j0 <= rp->n_p + 1; j0 += L.tile_j) tiles.push_back({pi, i0, j0});
                    pi++;
                }
    L.ntiles = (int)tiles.size();
    P.put(L.dtiles, tiles);
    if (L.precision == kF32) {  // strip tiles of the fused face + flux kernels
        std::vector<TileRef> xt, pt;
        pi = 0;
        for (Run *R : L.runs)
            for (auto &sp : R->rects)
                for (auto &lvl : sp)
                    for (auto &rp : lvl) {
                        for (int i0 = 0; i0 <= rp->n_x; i0 += kStripRows)
                            for (int j0 = -1; j0 <= rp->n_p; j0 += kXCols) xt.push_back({pi, i0, j0});
                        for (int i0 = -1; i0 <= rp->n_x; i0 += kStripRows)
                            for (int j0 = 0; j0 <= rp->n_p; j0 += 32) pt.push_back({pi, i0, j0});
                        pi++;
                    }
        L.nxtiles = (int)xt.size();
        L.nptiles = (int)pt.size();
        P.put(L.dxtiles, xt);
        P.put(L.dptiles, pt);
    }
    if (!pk) {  // rebuilt alone (the autotuner's trial shapes)
        L.tile_arena = DevBuf(alone.bytes(), DevBuf::Uninit{});
        alone.place(L.tile_arena);
        alone.copy(stream);
    }
}

// The set's host tables are packed into one allocation and copied, and its op tables
// gathered from the runs' own lists, by kernels queued on `stream`: ordered after the
// work already there (which may still be writing the runs' lists) and before any use, and
// never waited for on the host — a serving loop builds the next step's set while the
// current step runs.
// The set's host tables are packed into one allocation; flush_set then copies them and
// gathers its op tables from the runs' own lists, by kernels queued on `stream` — after
// the work already there (which may still be writing the runs' lists) and before any use.
// A serving loop builds the next step's set on the host while the current step runs and
// queues the copies once it is done (a launch queued behind a running step's graph holds
// the host up).
void Engine::build_set(LaunchSet &L) {
    // VX_TRACE_INIT=1: host time of each phase on stderr
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char *what) {
        if (!trace) return;
        auto t1 = std::chrono::steady_clock::now();
        std::fprintf(stderr, "vx set %-12s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
    L.precision = L.runs.empty() ? kF64 : L.runs[0]->precision;
    L.tile_j = tile_pref[L.precision == kF32][0];
    L.tile_i = tile_pref[L.precision == kF32][1];
    L.poisson = L.runs.empty() ? kPoissonLU : L.runs[0]->poisson;
    L.fast64 = L.runs.empty() ? 0 : L.runs[0]->fast64;
    for (Run *R : L.runs) {
        if (R->precision != L.precision)
            throw std::invalid_argument("runs advanced together must share one precision");
        if (R->poisson != L.poisson)
            throw std::invalid_argument("runs advanced together must share one Poisson solver");
        if (R->fast64 != L.fast64)
            throw std::invalid_argument("runs advanced together must share one FP64 kernel form");
    }
    L.pending_pack.reset(new TablePack);  // every table below: one allocation, one copy
    TablePack &pk = *L.pending_pack;
    std::vector<PoissonFastDev> pfs;
    for (Run *R : L.runs) pfs.push_back(R->pfdev);
    pk.put(L.dpf, pfs);
    std::vector<int> colpatch, colidx, lvl_ptr, lvl_off, lvl_patch, run_n, run_ns, run_nl;
    std::vector<RunFields> fields;
    std::vector<LUDev> lus;
    std::vector<double> dxinv, spec;
    L.hpatch.clear();
    L.maxnp = 0;
    L.maxn = 0;
    L.maxnf = 0;
    for (size_t ri = 0; ri < L.runs.size(); ri++) {
        Run &R = *L.runs[ri];
        const Settings &s = *R.S;
        int ns = (int)R.rects.size(), nl = s.maxDepth + 1;
        lvl_off.push_back((int)lvl_ptr.size());
        std::vector<int> ptr;
        ptr.push_back((int)lvl_patch.size());  // absolute: this run's first patch
        for (int sp = 0; sp < ns; sp++) {
            for (int l = 0; l < nl; l++) {
                for (auto &rp : R.rects[sp][l]) {
                    Rect &r = *rp;
                    R.upload_rect_desc(r, (int)ri);
                    int pi = (int)L.hpatch.size();
                    L.hpatch.push_back(r.desc);
                    lvl_patch.push_back(pi);
                    int rtb = r.desc.rtb;
                    // one moment column per coarse column (the kernels form its rtb
                    // finest sub-columns from shared loads); c = i * rtb
                    for (int c = 0; c < r.n_x * rtb; c += rtb) {
                        colpatch.push_back(pi);
                        colidx.push_back(c);
                    }
                    // FP64: blocks of kMomCols columns of one patch (padding: patch -1)
                    if (L.precision == kF64)
                        while (colpatch.size() % kMomCols) {
                            colpatch.push_back(-1);
                            colidx.push_back(0);
                        }
                    L.maxnp = std::max(L.maxnp, r.n_p);
                }
                ptr.push_back((int)lvl_patch.size());
            }
        }
        // lvl_ptr entries are absolute indices into lvl_patch
        for (int v : ptr) lvl_ptr.push_back(v);
        run_n.push_back(R.n);
        run_ns.push_back(ns);
        run_nl.push_back(nl);
        fields.push_back(R.F);
        lus.push_back(R.ludev);
        dxinv.push_back(1 / s.GetDx(0));
        L.w.push_back(std::pow(s.GetDx(0), 2.0));
        L.fcoef.push_back(1.0 / (12 * s.GetDx(0)));
        L.maxn = std::max(L.maxn, R.n);
        L.maxnf = std::max(L.maxnf, R.nf);
        // CFL species table (EMSolver.cpp:631-646)
        std::vector<double> sp(25, 0.0);
        double dpsMax(0.0);
        for (int i = 0; i < ns && i < 8; i++) {
            double dps = 1 / s.GetDp(0, i);
            dpsMax = std::max(dpsMax, std::fabs(s.q[i]) * dps);
            sp[3 * i] = std::fabs(s.q[i]);
            sp[3 * i + 1] = s.m[i];
            sp[3 * i + 2] = dps;
        }
        sp[24] = dpsMax;
        spec.insert(spec.end(), sp.begin(), sp.end());
    }
    lap("runs");
    // AMR op tables: batch b of the set = batch b of every run, patch ids made global.
    // Each run's sorted lists already sit on the device; the set's tables are gathered
    // there, one segment per (batch, run), so a new set costs no host-side op copies.
    // The segment lists go into the pack; the gathers run once it is on the device.
    std::vector<std::function<void()>> &gathers = L.pending_gathers;
    gathers.clear();
    DevBuf *dsegs = L.dsegs;
    {
        int which = 0;
        auto gather = [&](auto dummy, auto table_of, auto ptr_of, auto merge, DevBuf &out, std::vector<int> &optr) {
            using Op = decltype(dummy);
            size_t nb = 0;
            for (Run *R : L.runs) nb = std::max(nb, ptr_of(*R).empty() ? (size_t)0 : ptr_of(*R).size() - 1);
            std::vector<OpSegment> segs;
            optr.assign(1, 0);
            long long total = 0;
            for (size_t bt = 0; bt < nb; bt++) {
                int base = 0;
                for (Run *R : L.runs) {
                    const std::vector<int> &p = ptr_of(*R);
                    if (bt + 1 < p.size() && p[bt + 1] > p[bt]) {
                        const int cnt = p[bt + 1] - p[bt];
                        segs.push_back({table_of(*R).template as<Op>() + p[bt], total, cnt, base});
                        total += cnt;
                    }
                    base += (int)R->flat.size();
                }
                optr.push_back((int)total);
            }
            pk.reserve(out, (size_t)std::max<long long>(total, 1) * sizeof(Op));
            DevBuf &ds = dsegs[which++];
            const int nseg = (int)segs.size();
            if (nseg) {
                pk.put(ds, segs);
                gathers.push_back([&ds, &out, nseg, merge, this] { merge(ds.as<OpSegment>(), nseg, out.as<Op>(), stream); });
            }
        };
        gather(GhostOp{}, [](Run &R) -> DevBuf & { return R.dghost_ops; },
               [](Run &R) -> const std::vector<int> & { return R.ghost_b.ptr; }, merge_ghost_ops, L.dghost,
               L.ghost_ptr);
        gather(IfaceOp{}, [](Run &R) -> DevBuf & { return R.diface_ops; },
               [](Run &R) -> const std::vector<int> & { return R.iface_b.ptr; }, merge_iface_ops, L.diface,
               L.iface_ptr);
        gather(CSyncOp{}, [](Run &R) -> DevBuf & { return R.dcsync_ops; },
               [](Run &R) -> const std::vector<int> & { return R.csync_b.ptr; }, merge_csync_ops, L.dcsync,
               L.csync_ptr);
        L.max_batch = 0;
        for (const std::vector<int> *p : {&L.ghost_ptr, &L.iface_ptr, &L.csync_ptr})
            for (size_t b = 0; b + 1 < p->size(); b++) L.max_batch = std::max(L.max_batch, (*p)[b + 1] - (*p)[b]);
        pk.put(L.dghost_ptr, L.ghost_ptr);
        pk.put(L.diface_ptr, L.iface_ptr);
        pk.put(L.dcsync_ptr, L.csync_ptr);
    }
    lap("op tables");
    // Moment work units (FP64: blocks of kMomCols columns of one patch; FP32: one column
    // per warp) longest first: a unit's time grows with its patch's n_p and sub-columns,
    // and the GPU schedules blocks in list order, so the short units of the fine levels
    // fill the tail instead of leaving a last wave of long base-level blocks alone on a
    // few SMs.  Each column's result is independent of the order.
    {
        // A unit's cost depends on its patch alone and a patch's units are consecutive in
        // the list, so a stable sort of the patches' unit ranges by cost gives the stable
        // sort of the units (in O(units) instead of sorting every unit).
        const int unit = L.precision == kF64 ? kMomCols : 1;
        const int nunits = (int)colpatch.size() / unit;
        struct Range {
            int u0, u1;
            long long cost;
        };
        std::vector<Range> ranges;
        for (int u = 0; u < nunits;) {
            const int pi = colpatch[(size_t)u * unit];
            int u1 = u + 1;
            while (u1 < nunits && colpatch[(size_t)u1 * unit] == pi) u1++;
            const PatchT<double> &d = L.hpatch[pi];
            ranges.push_back({u, u1, (long long)(d.np + 2) * ((d.rtb + 1) / 2)});
            u = u1;
        }
        std::stable_sort(ranges.begin(), ranges.end(), [](const Range &a, const Range &b) { return a.cost > b.cost; });
        std::vector<int> cp2, ci2;
        cp2.reserve(colpatch.size());
        ci2.reserve(colidx.size());
        for (const Range &rg : ranges) {
            cp2.insert(cp2.end(), colpatch.begin() + (size_t)rg.u0 * unit, colpatch.begin() + (size_t)rg.u1 * unit);
            ci2.insert(ci2.end(), colidx.begin() + (size_t)rg.u0 * unit, colidx.begin() + (size_t)rg.u1 * unit);
        }
        colpatch.swap(cp2);
        colidx.swap(ci2);
    }
    L.ncols = (int)colpatch.size();
    build_pipe_tables(L, colpatch, colidx, pk);
    lap("units");
    // lvl_ptr is absolute; lvl_off points at each run's block.
    pk.put(L.dpatch, L.hpatch);
    build_tiles(L, &pk);
    lap("tiles");
    pk.put(L.dfields, fields);
    pk.put(L.dcolpatch, colpatch);
    pk.put(L.dcolidx, colidx);
    pk.put(L.dlvl_ptr, lvl_ptr);
    pk.put(L.dlvl_off, lvl_off);
    pk.put(L.dlvl_patch, lvl_patch);
    pk.put(L.drun_n, run_n);
    pk.put(L.drun_ns, run_ns);
    pk.put(L.drun_nl, run_nl);
    pk.put(L.dlu, lus);
    pk.put(L.dw, L.w);
    pk.put(L.dfcoef, L.fcoef);
    pk.put(L.ddxinv, dxinv);
    pk.put(L.dcfl_spec, spec);
    pk.put(L.dns, run_ns);
    pk.put(L.dcfl_out, std::vector<double>(L.runs.size(), 0.0));
    L.hparams.assign(L.runs.size() * 6 * kParamStride, 0.0);
    pk.put(L.dparams, L.hparams);
    L.hparams32.assign(L.hparams.size(), 0.0f);
    pk.put(L.dparams32, L.hparams32);
    lap("tables");
    L.arena = take_arena(pk.bytes());
    pk.place(L.arena);  // the views are final: a graph can be captured from here on
    if (L.graph) {
        cudaGraphExecDestroy(L.graph);
        L.graph = nullptr;
    }
    lap("arena");
}

// The set's table copy and op gathers, queued on `stream` (once).
void Engine::flush_set(LaunchSet &L) {
    if (!L.pending_pack) return;
    // the staging is reused once the previous set's copy has run
    VX_CUDA(cudaEventSynchronize(ev_pinned_));
    TablePack &pk = *L.pending_pack;
    pk.copy(stream, pinned_staging(pk.staged_bytes()), pinned_dev_);
    VX_CUDA(cudaEventRecord(ev_pinned_, stream));
    for (auto &g : L.pending_gathers) g();
    L.pending_gathers.clear();
    L.pending_pack.reset();
}

void Engine::flush_prepared() {
    for (auto &kv : sets_) flush_set(*kv.second);
}

// Tables of the pipelined moments + solve launch (k64_moments_poisson) for an FP64 set
// with the exact solve: the moment units in the order the forward sweeps first need their
// columns, the done counter each unit adds to, and per run and forward chunk the rows
// whose right-hand side the chunk reads first.  A unit covers finest x positions
// [(x_pos * rtb) + c, ... + rtb) for each of its columns c = i * rtb; row k's right-hand
// side comes from position perm[k].
void Engine::build_pipe_tables(LaunchSet &L, const std::vector<int> &colpatch, const std::vector<int> &colidx,
                               TablePack &pk) {
    L.pipe = false;
    if (L.precision != kF64 || L.poisson != kPoissonLU || L.runs.empty() || (int)L.runs.size() > kPipeMaxRuns) return;
    for (Run *R : L.runs)
        if (R->pipe_rfc.empty() || (int)R->pipe_rfc.size() != R->n) return;
    const int R = kPoisRowsHost;
    std::vector<int> run_ctr, run_gptr, gptr, grow, need;
    std::vector<std::vector<int>> xfc(L.runs.size());  // per run and x position: first chunk needing it
    for (size_t ri = 0; ri < L.runs.size(); ri++) {
        const Run &Rn = *L.runs[ri];
        const int n = Rn.n, nch = (n + R - 1) / R;
        run_ctr.push_back((int)need.size());
        need.resize(need.size() + nch, 0);
        xfc[ri].assign(n, 0);
        for (int k = 0; k < n; k++) xfc[ri][Rn.lu.perm[k]] = Rn.pipe_rfc[k];
        // rows grouped by the chunk that reads them first, ascending within a chunk
        run_gptr.push_back((int)gptr.size());
        std::vector<int> cnt(nch + 1, 0);
        for (int k = 0; k < n; k++) cnt[Rn.pipe_rfc[k] + 1]++;
        for (int c = 0; c < nch; c++) cnt[c + 1] += cnt[c];
        const int base = (int)grow.size();
        for (int c = 0; c <= nch; c++) gptr.push_back(base + cnt[c]);
        grow.resize(base + n);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int k = 0; k < n; k++) grow[base + fill[Rn.pipe_rfc[k]]++] = k;
    }
    const int nunits = (int)colpatch.size() / kMomCols;
    std::vector<int> ufc(nunits, 0), urun(nunits, 0);
    for (int u = 0; u < nunits; u++) {
        const PatchT<double> &P = L.hpatch[colpatch[(size_t)u * kMomCols]];
        const int ri = P.run;
        const std::vector<int> &xf = xfc[ri];
        int fc = INT32_MAX;
        for (int w = 0; w < kMomCols; w++) {
            if (colpatch[(size_t)u * kMomCols + w] < 0) continue;
            const int x0 = P.x_pos * P.rtb + colidx[(size_t)u * kMomCols + w];
            for (int k = 0; k < P.rtb; k++) {
                const int x = x0 + k;
                if (x < 0 || x >= (int)xf.size()) return;  // not a layout the pipelined form covers
                fc = std::min(fc, xf[x]);
            }
        }
        if (fc == INT32_MAX) return;
        ufc[u] = fc;
        urun[u] = ri;
    }
    // units by first needed chunk (then the longest-first order they already have); a
    // unit's items (p windows of each sub-column pair) are consecutive tickets
    std::vector<int> order(nunits);
    for (int u = 0; u < nunits; u++) order[u] = u;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ufc[a] < ufc[b]; });
    std::vector<int> col0(nunits), sig(nunits), item0(nunits + 1, 0), nwin(nunits), item_unit;
    std::vector<double2> c12(nunits);
    for (int t = 0; t < nunits; t++) {
        const int u = order[t];
        const PatchT<double> &P = L.hpatch[colpatch[(size_t)u * kMomCols]];
        col0[t] = u * kMomCols;
        sig[t] = run_ctr[urun[u]] + ufc[u];
        need[sig[t]]++;
        nwin[t] = (P.np + kMomWindow - 1) / kMomWindow;
        const int items = (P.rtb + 1) / 2 * nwin[t];
        item0[t + 1] = item0[t] + items;
        item_unit.insert(item_unit.end(), items, t);
        // the moments' (1 / m) / c and its reciprocal, in their operations
        const double minv = 1 / P.mass;
        const double c1 = minv * kCInv;
        c12[t] = make_double2(c1, 1 / c1);
    }
    const int nitems = item0[nunits];
    if ((size_t)nitems * kPipeItemDoubles * sizeof(double) > kPipeMaxScratch) return;
    L.pipe_nunits = nunits;
    L.pipe_nitems = nitems;
    L.pipe_ndone = (int)need.size();
    pk.put(L.dpipe_col0, col0);
    pk.put(L.dpipe_sig, sig);
    pk.put(L.dpipe_item0, item0);
    pk.put(L.dpipe_nwin, nwin);
    pk.put(L.dpipe_c12, c12);
    pk.put(L.dpipe_items, item_unit);
    pk.put(L.dpipe_need, need);
    pk.put(L.dpipe_runctr, run_ctr);
    pk.put(L.dpipe_rungptr, run_gptr);
    pk.put(L.dpipe_gptr, gptr);
    pk.put(L.dpipe_grow, grow);
    L.dpipe_scratch = DevBuf((size_t)nitems * kPipeItemDoubles * sizeof(double));
    L.dpipe_state = DevBuf((size_t)(kPipeDone + L.pipe_ndone + 2 * nunits) * sizeof(unsigned));  // zeroed
    // summing warps, four per block: each unit's sums take about 64 cycles per FP64 add on
    // their sub-partition; enough blocks that they keep up with the column warps
    long long adds = 0;
    for (int t = 0; t < nunits; t++) adds += (long long)(item0[t + 1] - item0[t]) * 2 * kMomWindow;
    L.pipe_summers = (int)std::min<long long>(8, std::max<long long>(1, (adds * 64 / 4 + 1200000 - 1) / 1200000));
    if (!pipe_err_.p) pipe_err_ = DevBuf(sizeof(int));
    L.pipe = true;
}

// Launch descriptors of a set's step kernels (tables, tiles, fields, parameter blocks).
StageLaunches Engine::stage_launches(LaunchSet &L) {
    StageLaunches K{};
    FctLaunch &fl = K.fl;
    MomLaunch &ml = K.ml;
    AsmLaunch &al = K.al;
    PoissonLaunch &pl = K.pl;
    MaxwellLaunch &mx = K.mx;
    fl.patches = L.dpatch.p;
    fl.tiles = L.dtiles.as<TileRef>();
    fl.ntiles = L.ntiles;
    fl.tile_j = L.tile_j;
    fl.tile_i = L.tile_i;
    fl.xtiles = L.dxtiles.as<TileRef>();
    fl.ptiles = L.dptiles.as<TileRef>();
    fl.nxtiles = L.nxtiles;
    fl.nptiles = L.nptiles;
    fl.fields = L.dfields.as<RunFields>();
    fl.params = L.dparams.as<double>();
    fl.params32 = L.dparams32.as<float>();
    fl.use_f0 = 0;
    fl.stream = stream;
    ml.patches = L.dpatch.p;
    ml.colpatch = L.dcolpatch.as<int>();
    ml.colidx = L.dcolidx.as<int>();
    ml.ncols = L.ncols;
    ml.maxnp = L.maxnp;
    ml.fields = L.dfields.as<RunFields>();
    ml.nruns = (int)L.runs.size();
    ml.maxnf = L.maxnf;
    ml.fast = L.precision == kF64 ? L.fast64 : 0;
    ml.stream = stream;
    al.patches = L.dpatch.p;
    al.lvl_ptr = L.dlvl_ptr.as<int>();
    al.lvl_off = L.dlvl_off.as<int>();
    al.lvl_patch = L.dlvl_patch.as<int>();
    al.run_n = L.drun_n.as<int>();
    al.run_ns = L.drun_ns.as<int>();
    al.run_nl = L.drun_nl.as<int>();
    al.nruns = (int)L.runs.size();
    al.maxn = L.maxn;
    al.pairs = L.precision == kF32 ? 1 : 0;
    al.fields = L.dfields.as<RunFields>();
    al.stream = stream;
    pl.lu = L.dlu.as<LUDev>();
    pl.fields = L.dfields.as<RunFields>();
    pl.w = L.dw.as<double>();
    pl.fcoef = L.dfcoef.as<double>();
    pl.nruns = (int)L.runs.size();
    pl.maxn = L.maxn;
    pl.stream = stream;
    mx.fields = L.dfields.as<RunFields>();
    mx.nruns = (int)L.runs.size();
    mx.maxnf = L.maxnf;
    mx.params = L.dparams.as<double>();
    mx.dxinv = L.ddxinv.as<double>();
    mx.f32 = L.precision == kF32;
    mx.stream = stream;
    return K;
}

// The kernel sequence of one full RK step (SolverManager.cpp:28-39 -> Mesh.cpp:64-89,
// EMSolver.cpp:104-202) for every run of the set.
void Engine::record_step(LaunchSet &L) {
    if (persistent && L.precision == kF32) {
        record_step_persistent32(L);
        return;
    }
    int launches = 0;
    StageLaunches K = stage_launches(L);
    FctLaunch &fl = K.fl;
    MomLaunch &ml = K.ml;
    AsmLaunch &al = K.al;
    PoissonLaunch &pl = K.pl;
    MaxwellLaunch &mx = K.mx;
    const bool pipe = pipelined && L.pipe;
    for (int s = 0; s < 6; s++) {
        if (pipe) {
            record_pipe_stage(L, K, s, launches);
            continue;
        }
        // FP32 copies of the fields: E_x's comes with each solve (k_efield), the per-cell
        // A^2 the moments read with each Maxwell stage for the next one (the step's first
        // stage makes its own), a^2's with the moments at every stage (the Maxwell stage
        // runs beside the face kernels that read it, so it cannot write the copy).
        ml.acell = s == 0;
        run_moments(L, ml);
        launch_assemble(al);
        launches += (L.precision == kF32 && s == 0) ? 3 : 2;
        // the Poisson solve (and E_x) runs beside the x-direction face work, which does
        // not read E_x; the p-direction faces wait for both
        VX_CUDA(cudaEventRecord(ev_fork, stream));
        VX_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
        pl.stream = side;
        run_poisson(L, pl);
        launches += 1;  // the scan solve forms E_x itself
        fl.step = s;
        // The Maxwell stage (EMFieldSolver::RGKStep) writes A and a^2, which the Vlasov
        // stage reads only in the gamma kernel (FP64) or the FP32 copy of a^2 made above;
        // it runs on the side stream after the Poisson solve, beside the rest of the FCT
        // chain, and joins before the next stage's moments.
        if (L.precision == kF64) {
            fct_sub(L, fl, kSubGamma);
            launches += 1;
        }
        VX_CUDA(cudaEventRecord(ev_join, side));
        VX_CUDA(cudaEventRecord(ev_gamma, stream));
        VX_CUDA(cudaStreamWaitEvent(side, ev_gamma, 0));
        mx.step = s;
        mx.stream = side;
        launch_maxwell(mx);
        launches += 3;
        VX_CUDA(cudaEventRecord(ev_mx, side));
        if (L.precision == kF32) {  // fused face + flux kernels per direction
            fct_sub(L, fl, kSubXFlux);
            VX_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
            fct_sub(L, fl, kSubPFlux);
            launches += 2;
        } else if (L.poisson == kPoissonLU) {
            // x faces and fluxes, and the E_x-independent half of the p faces, beside the
            // exact Poisson solve; then the p-face velocities (E_x) and the p fluxes
            fl.part = 1;
            fct_sub(L, fl, kSubFaces);
            fct_sub(L, fl, kSubFlux);
            fl.part = 4;
            fct_sub(L, fl, kSubFaces);
            VX_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
            fl.part = 8;
            fct_sub(L, fl, kSubFaces);
            fl.part = 2;
            fct_sub(L, fl, kSubFlux);
            fl.part = 0;
            launches += 5;
        } else {  // the scan solve is short: the p faces in one pass after it
            fl.part = 1;
            fct_sub(L, fl, kSubFaces);
            fct_sub(L, fl, kSubFlux);
            VX_CUDA(cudaStreamWaitEvent(stream, ev_join, 0));
            fl.part = 2;
            fct_sub(L, fl, kSubFaces);
            fct_sub(L, fl, kSubFlux);
            fl.part = 0;
            launches += 4;
        }
        for (size_t b = 0; b + 1 < L.iface_ptr.size(); b++, launches++)
            launch_iface(L.dpatch.p, L.diface.as<IfaceOp>() + L.iface_ptr[b], L.iface_ptr[b + 1] - L.iface_ptr[b], s, L.precision, stream);
        fct_sub(L, fl, kSubDsF2);
        launches += 1;
        for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
            launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 2, L.precision, stream);
        fct_sub(L, fl, kSubLimR);
        fct_sub(L, fl, kSubLimC);
        launches += 2;
        for (size_t b = 0; b + 1 < L.csync_ptr.size(); b++, launches++)
            launch_csync(L.dpatch.p, L.dcsync.as<CSyncOp>() + L.csync_ptr[b], L.csync_ptr[b + 1] - L.csync_ptr[b], L.precision, stream);
        fct_sub(L, fl, kSubUpdate);
        launches += 1;
        for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
            launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 1, L.precision, stream);
        if (s == 5) {
            fct_sub(L, fl, kSubCopy10);
            launches += 1;
        }
        VX_CUDA(cudaStreamWaitEvent(stream, ev_mx, 0));
    }
    L.launches_per_step = launches;
    if (pipe) pipe_pending_ = true;
}

// One RK stage of an FP64 exact-solve set in the pipelined form.  Main stream: the
// moments + solve launch, then (once the faces beside it are done) the E_x-dependent half
// of the p faces and the rest of the FCT chain.  Side stream, beside the launch: gamma, the
// x faces and fluxes and the E_x-independent half of the p faces (none reads rho, J or
// E_x), then the Maxwell stage after the launch (it reads J and rewrites A, which gamma
// reads).  The launch carries the highest stream priority, so its moment blocks go ahead
// of the face blocks and the solve's inputs arrive as early as possible.
PipeLaunch Engine::pipe_launch(LaunchSet &L, const StageLaunches &K) {
    PipeLaunch P{};
    P.M = K.ml;
    P.A = K.al;
    P.P = K.pl;
    P.P.stream = stream;
    P.unit_col0 = L.dpipe_col0.as<int>();
    P.unit_sig = L.dpipe_sig.as<int>();
    P.unit_item0 = L.dpipe_item0.as<int>();
    P.unit_nwin = L.dpipe_nwin.as<int>();
    P.unit_c12 = L.dpipe_c12.as<double2>();
    P.nunits = L.pipe_nunits;
    P.item_unit = L.dpipe_items.as<int>();
    P.nitems = L.pipe_nitems;
    P.scratch = L.dpipe_scratch.as<double>();
    P.summers = L.pipe_summers;
    P.workers = std::max(1, std::min(num_sms_ - (int)L.runs.size() - P.summers, (L.pipe_nitems + 1) / 2));
    P.need = L.dpipe_need.as<int>();
    P.ndone = L.pipe_ndone;
    P.run_ctr = L.dpipe_runctr.as<int>();
    P.run_gptr = L.dpipe_rungptr.as<int>();
    P.gptr = L.dpipe_gptr.as<int>();
    P.grow = L.dpipe_grow.as<int>();
    P.state = L.dpipe_state.as<unsigned>();
    P.err = pipe_err_.as<int>();
    P.limit_ns = persist_limit_ns;
    P.phantom = persist_phantom;
    P.priority = prio_hi_;
    P.stream = stream;
    return P;
}

void Engine::record_pipe_stage(LaunchSet &L, StageLaunches &K, int s, int &launches) {
    FctLaunch &fl = K.fl;
    MaxwellLaunch &mx = K.mx;
    const PipeLaunch P = pipe_launch(L, K);
    VX_CUDA(cudaEventRecord(ev_fork, stream));
    VX_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
    launch_moments_poisson64(P);
    VX_CUDA(cudaEventRecord(ev_join, stream));
    fl.step = s;
    fl.stream = side;
    fct_sub(L, fl, kSubGamma);
    fl.part = 1;
    fct_sub(L, fl, kSubFaces);
    fct_sub(L, fl, kSubFlux);
    fl.part = 4;
    fct_sub(L, fl, kSubFaces);
    VX_CUDA(cudaEventRecord(ev_gamma, side));
    VX_CUDA(cudaStreamWaitEvent(side, ev_join, 0));
    mx.step = s;
    mx.stream = side;
    launch_maxwell(mx);
    VX_CUDA(cudaEventRecord(ev_mx, side));
    launches += 1 + 4 + 3;
    fl.stream = stream;
    VX_CUDA(cudaStreamWaitEvent(stream, ev_gamma, 0));
    fl.part = 8;
    fct_sub(L, fl, kSubFaces);
    fl.part = 2;
    fct_sub(L, fl, kSubFlux);
    fl.part = 0;
    launches += 2;
    for (size_t b = 0; b + 1 < L.iface_ptr.size(); b++, launches++)
        launch_iface(L.dpatch.p, L.diface.as<IfaceOp>() + L.iface_ptr[b], L.iface_ptr[b + 1] - L.iface_ptr[b], s, L.precision, stream);
    fct_sub(L, fl, kSubDsF2);
    launches += 1;
    for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
        launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 2, L.precision, stream);
    fct_sub(L, fl, kSubLimR);
    fct_sub(L, fl, kSubLimC);
    launches += 2;
    for (size_t b = 0; b + 1 < L.csync_ptr.size(); b++, launches++)
        launch_csync(L.dpatch.p, L.dcsync.as<CSyncOp>() + L.csync_ptr[b], L.csync_ptr[b + 1] - L.csync_ptr[b], L.precision, stream);
    fct_sub(L, fl, kSubUpdate);
    launches += 1;
    for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
        launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 1, L.precision, stream);
    if (s == 5) {
        fct_sub(L, fl, kSubCopy10);
        launches += 1;
    }
    VX_CUDA(cudaStreamWaitEvent(stream, ev_mx, 0));
}

void Engine::set_pipelined(bool on) {
    sync();
    pipelined = on;
    for (auto &kv : sets_)
        if (kv.second->graph) {
            cudaGraphExecDestroy(kv.second->graph);
            kv.second->graph = nullptr;
        }
}

// The persistent form of an FP32 set's step: per RK stage the moments and assembly in
// one cooperative launch, the Poisson solve, then the FCT stage with the Maxwell stage
// beside it in a second cooperative launch (stage32.cu) — three launches per stage, in
// stream order (the solve no longer overlaps the x-direction fluxes: they share the
// second launch with the p-direction ones).
void Engine::record_step_persistent32(LaunchSet &L) {
    if (!gsync_.p) throw std::logic_error("persistent form recorded without its barrier state");
    StageLaunches K = stage_launches(L);
    Stage32Launch S{};
    S.fl = K.fl;
    S.ml = K.ml;
    S.al = K.al;
    S.mx = K.mx;
    S.mx.asq32_out = 1;  // the next stage's x fluxes run beside its moments (see launch_stage32_pre)
    S.ghost = L.dghost.as<GhostOp>();
    S.ghost_ptr = L.dghost_ptr.as<int>();
    S.nghost_b = L.ghost_ptr.empty() ? 0 : (int)L.ghost_ptr.size() - 1;
    S.iface = L.diface.as<IfaceOp>();
    S.iface_ptr = L.diface_ptr.as<int>();
    S.niface_b = L.iface_ptr.empty() ? 0 : (int)L.iface_ptr.size() - 1;
    S.csync = L.dcsync.as<CSyncOp>();
    S.csync_ptr = L.dcsync_ptr.as<int>();
    S.ncsync_b = L.csync_ptr.empty() ? 0 : (int)L.csync_ptr.size() - 1;
    S.max_batch = L.max_batch;
    S.sync = gsync_.as<GridSyncState>();
    S.limit_ns = persist_limit_ns;
    S.phantom = persist_phantom;
    S.stream = stream;
    PoissonLaunch pl = K.pl;
    pl.stream = stream;
    unsigned long long *tr = stage_trace_.as<unsigned long long>();
    for (int s = 0; s < 6; s++) {
        S.step = s;
        S.fl.step = s;
        S.mx.step = s;
        S.ml.acell = s == 0;
        S.trace = tr ? tr + (2 * s) * kStageTraceSlots : nullptr;
        launch_stage32_pre(S);
        run_poisson(L, pl);
        S.trace = tr ? tr + (2 * s + 1) * kStageTraceSlots : nullptr;
        launch_stage32_fct(S);
    }
    L.launches_per_step = 18;
    gsync_pending_ = true;
}

void Engine::set_persistent(bool on) {
    sync();
    if (on && !gsync_.p) gsync_ = DevBuf(sizeof(GridSyncState));  // zeroed; not during a capture
    if (on && !stage_trace_.p && std::getenv("VX_TRACE_STAGE"))
        stage_trace_ = DevBuf(12 * kStageTraceSlots * sizeof(unsigned long long));
    persistent = on;
    for (auto &kv : sets_)
        if (kv.second->graph) {
            cudaGraphExecDestroy(kv.second->graph);
            kv.second->graph = nullptr;
        }
}

void Engine::set_persistent_limit(unsigned long long limit_ns, int phantom) {
    if (limit_ns == 0 || phantom < 0) throw std::invalid_argument("persistent barrier limit must be > 0, phantom >= 0");
    set_persistent(persistent);  // the captured graphs hold the old values
    persist_limit_ns = limit_ns;
    persist_phantom = phantom;
}

void Engine::check_device_errors() {
    if (pipe_pending_ && pipe_err_.p) {
        pipe_pending_ = false;
        int e = 0;
        VX_CUDA(cudaMemcpy(&e, pipe_err_.p, sizeof e, cudaMemcpyDeviceToHost));
        if (e != 0) {
            VX_CUDA(cudaMemset(pipe_err_.p, 0, sizeof(int)));
            throw TimeoutError("pipelined moments + Poisson solve: the wait for the moments of done counter " +
                               std::to_string(e - 1) + " ran out (the step's results are not valid)");
        }
    }
    if (!gsync_pending_ || !gsync_.p) return;
    gsync_pending_ = false;
    if (stage_trace_.p) {  // per launch: each phase's work (to its last arrival) and the barrier's release
        std::vector<unsigned long long> t(12 * kStageTraceSlots);
        VX_CUDA(cudaMemcpy(t.data(), stage_trace_.p, t.size() * sizeof(t[0]), cudaMemcpyDeviceToHost));
        for (int l = 0; l < 12; l++) {
            const unsigned long long *q = &t[(size_t)l * kStageTraceSlots];
            std::fprintf(stderr, "vx stage %d %s:", l / 2, l % 2 ? "fct" : "pre");
            unsigned long long prev = q[0];
            for (int k = 1; 2 * k < kStageTraceSlots; k++) {
                const unsigned long long arr = q[2 * k - 1], ex = q[2 * k];
                if (arr < prev || arr == 0) break;
                std::fprintf(stderr, " %.1f", (arr - prev) * 1e-3);
                if (ex < arr) break;  // the launch's end (no barrier after its last phase)
                std::fprintf(stderr, "+%.1f", (ex - arr) * 1e-3);
                prev = ex;
            }
            std::fprintf(stderr, " us\n");
        }
    }
    GridSyncState h{};
    VX_CUDA(cudaMemcpy(&h, gsync_.p, sizeof h, cudaMemcpyDeviceToHost));
    if (h.err != 0) {
        VX_CUDA(cudaMemset(gsync_.p, 0, sizeof(GridSyncState)));
        throw TimeoutError("persistent stage kernel: the wait at grid barrier " + std::to_string(h.err) +
                           " ran out (the step's results are not valid)");
    }
}

// The dt-scaled weights of RK stage st: FCT [0..5] and their left-to-right sum [6] (as
// Rectangle.cpp:1396-1517 forms aSum), Maxwell [8..13] (EMSolver.cpp:204-338, the last
// stage with b - a_4).  The laser entries [16], [17] are left to the caller.
static void stage_weights(double *p, int st, double timestep) {
    for (int k = 0; k < kParamStride; k++) p[k] = 0.0;
    if (st < 5) {
        for (int k = 0; k <= st; k++) p[k] = kRK[st][k] * timestep;
        double sum = p[0];
        for (int k = 1; k <= st; k++) sum = sum + p[k];
        p[6] = sum;
    } else {
        for (int k = 0; k < 6; k++) p[k] = kRK[5][k] * timestep;
        double sum = p[0];
        for (int k = 1; k < 6; k++) sum = sum + p[k];
        p[6] = sum;
    }
    if (st < 5) {
        for (int k = 0; k <= st; k++) p[8 + k] = kRK[st][k] * timestep;
    } else {
        double a[6];
        for (int k = 0; k < 5; k++) a[k] = kRK[4][k] * timestep;
        a[5] = 0;
        for (int k = 0; k < 6; k++) p[8 + k] = kRK[5][k] * timestep - a[k];
    }
}

// Host-side stage parameters (dt-scaled tableau, laser boundary values) of one step of
// every run of the set; advances each run's time through Settings::UpdateTime.
void Engine::fill_params(LaunchSet &L, const std::vector<Run *> &set, const std::vector<double> &dt) {
    for (size_t ri = 0; ri < set.size(); ri++) {
        Run &R = *set[ri];
        Settings &s = *R.S;
        double timestep = dt[ri];
        for (int st = 0; st < 6; st++) {
            double *p = &L.hparams[param_base((int)ri, st)];
            stage_weights(p, st, timestep);
            s.UpdateTime(st, timestep);
            p[16] = s.GetBY(0, s.time);
            p[17] = s.GetBZ(0, s.time);
        }
    }
    VX_CUDA(cudaMemcpyAsync(L.dparams.p, L.hparams.data(), L.hparams.size() * sizeof(double), cudaMemcpyHostToDevice,
                            stream));
    if (L.precision == kF32) {
        for (size_t q = 0; q < L.hparams.size(); q++) L.hparams32[q] = (float)L.hparams[q];
        VX_CUDA(cudaMemcpyAsync(L.dparams32.p, L.hparams32.data(), L.hparams32.size() * sizeof(float),
                                cudaMemcpyHostToDevice, stream));
    }
}

// Selected phases of RK stage s of one run, launched one after another on the context
// stream (no graph, no side stream): the per-class entry points.  The kernels and their
// order are those of record_step, so a step composed of these calls in the reference's
// order (SolverManager.cpp:28-39) gives the same bits as Engine::advance.
void Engine::run_phases(Run &run, int s, double dt, unsigned phases) {
    if (s < 0 || s > 5) throw std::invalid_argument("stage must be in 0..5");
    LaunchSet &L = get_set({&run});
    if (phases & (kPhSub0 | kPhMaxwell)) {
        double *p = &L.hparams[param_base(0, s)];
        stage_weights(p, s, dt);
        p[16] = run.S->GetBY(0, run.S->time);
        p[17] = run.S->GetBZ(0, run.S->time);
        VX_CUDA(cudaMemcpyAsync(L.dparams.as<double>() + param_base(0, s), p, kParamStride * sizeof(double),
                                cudaMemcpyHostToDevice, stream));
        if (L.precision == kF32) {
            float *q = &L.hparams32[param_base(0, s)];
            for (int k = 0; k < kParamStride; k++) q[k] = (float)p[k];
            VX_CUDA(cudaMemcpyAsync(L.dparams32.as<float>() + param_base(0, s), q, kParamStride * sizeof(float),
                                    cudaMemcpyHostToDevice, stream));
        }
        // the host copies are read by the asynchronous uploads; keep them until done
        sync();
    }
    StageLaunches K = stage_launches(L);
    FctLaunch &fl = K.fl;
    fl.step = s;
    int launches = 0;
    if (phases & kPhMoments) {  // EMFieldSolver::AssembleRhoAndJ
        K.ml.acell = 1;
        run_moments(L, K.ml);
        launch_assemble(K.al);
        launches += (L.precision == kF32) ? 3 : 2;
    }
    if (phases & kPhPoisson) {  // EMFieldSolver::UpdatePotential and E_x
        run_poisson(L, K.pl);
        launches += 1;
    }
    if (phases & kPhSub0) {  // Level::FCTTimeStep(dt, s, 0) coarsest first, incl. interface fluxes
        if (L.precision == kF32) {
            fct_sub(L, fl, kSubXFlux);
            fct_sub(L, fl, kSubPFlux);
            launches += 2;
        } else {
            fct_sub(L, fl, kSubGamma);
            fl.part = 0;
            fct_sub(L, fl, kSubFaces);
            fct_sub(L, fl, kSubFlux);
            launches += 3;
        }
        for (size_t b = 0; b + 1 < L.iface_ptr.size(); b++, launches++)
            launch_iface(L.dpatch.p, L.diface.as<IfaceOp>() + L.iface_ptr[b], L.iface_ptr[b + 1] - L.iface_ptr[b], s,
                         L.precision, stream);
        fct_sub(L, fl, kSubDsF2);
        launches += 1;
    }
    if (phases & kPhSub1) {  // PushData(2), FCTTimeStep(.., 1), PushBoundaryC
        for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
            launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 2,
                         L.precision, stream);
        fct_sub(L, fl, kSubLimR);
        fct_sub(L, fl, kSubLimC);
        launches += 2;
        for (size_t b = 0; b + 1 < L.csync_ptr.size(); b++, launches++)
            launch_csync(L.dpatch.p, L.dcsync.as<CSyncOp>() + L.csync_ptr[b], L.csync_ptr[b + 1] - L.csync_ptr[b],
                         L.precision, stream);
    }
    if (phases & kPhSub2) {  // FCTTimeStep(.., 2), PushData(1)
        fct_sub(L, fl, kSubUpdate);
        launches += 1;
        for (size_t b = 0; b + 1 < L.ghost_ptr.size(); b++, launches++)
            launch_ghost(L.dpatch.p, L.dghost.as<GhostOp>() + L.ghost_ptr[b], L.ghost_ptr[b + 1] - L.ghost_ptr[b], 1,
                         L.precision, stream);
    }
    if ((phases & kPhSub3) && s == 5) {  // FCTTimeStep(.., 3): Mesh::Advance runs it at the last stage only
        fct_sub(L, fl, kSubCopy10);
        launches += 1;
    }
    if (phases & kPhMaxwell) {  // EMFieldSolver::RGKStep
        K.mx.step = s;
        launch_maxwell(K.mx);
        launches += 3;
    }
    kernel_launches += launches;
    VX_CUDA(cudaGetLastError());
}

// The step of a set as one CUDA graph (its kernels read dt and the stage weights from the
// set's parameter block, so the graph serves every step).  Capturing only records: work
// already queued on the stream keeps running meanwhile.
void Engine::capture_graph(LaunchSet &L) {
    if (L.graph) return;
    static const bool trace = std::getenv("VX_TRACE_INIT") != nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    cudaGraph_t g;
    VX_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    record_step(L);
    VX_CUDA(cudaStreamEndCapture(stream, &g));
    const auto t1 = std::chrono::steady_clock::now();
    VX_CUDA(cudaGraphInstantiate(&L.graph, g, 0));
    cudaGraphDestroy(g);
    if (trace)
        std::fprintf(stderr, "vx set capture      %8.2f ms (instantiate %.2f ms)\n",
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                     std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count());
}

void Engine::prepare(const std::vector<Run *> &set) { get_set(set, true); }

void Engine::advance(const std::vector<Run *> &set, const std::vector<double> &dt) {
    LaunchSet &L = get_set(set);
    fill_params(L, set, dt);
    if (use_graphs) {
        capture_graph(L);
        VX_CUDA(cudaGraphLaunch(L.graph, stream));
    } else {
        record_step(L);
    }
    kernel_launches += L.launches_per_step;
    VX_CUDA(cudaGetLastError());
}

std::vector<double> Engine::calculate_dt(const std::vector<Run *> &set) {
    LaunchSet &L = get_set(set);
    CflLaunch cl{};
    cl.fields = L.dfields.as<RunFields>();
    cl.nruns = (int)set.size();
    cl.maxn = L.maxn;
    cl.spec = L.dcfl_spec.as<double>();
    cl.run_ns = L.dns.as<int>();
    cl.out = L.dcfl_out.as<double>();
    cl.stream = stream;
    launch_cfl(cl);
    kernel_launches += 1;
    std::vector<double> pc(set.size());
    VX_CUDA(cudaMemcpyAsync(pc.data(), L.dcfl_out.p, pc.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
    sync();
    std::vector<double> dt(set.size());
    for (size_t i = 0; i < set.size(); i++) {
        const Settings &s = *set[i]->S;
        double bound = 1.0 / std::max((kCs / s.GetDx(0) + pc[i]), 1e-40);
        dt[i] = s.cfl * bound;
    }
    return dt;
}

// E_x on the finest grid from the current phi and Ex0 (after a state was loaded).
void Engine::refresh_efield(Run &run) {
    LaunchSet &L = get_set({&run});
    launch_efield(L.dfields.as<RunFields>(), L.dfcoef.as<double>(), 1, L.maxn, L.precision == kF32, stream);
    kernel_launches += 1;
}

// Moments and rho/J assembly only (used for EnforceChargeNeutralization).
// SolverManager::AdvanceFields (SolverManager.cpp:41-46): the six Maxwell stages alone,
// with the current density left as it is.
void Engine::advance_fields(const std::vector<Run *> &set, const std::vector<double> &dt) {
    LaunchSet &L = get_set(set);
    fill_params(L, set, dt);
    MaxwellLaunch mx{};
    mx.fields = L.dfields.as<RunFields>();
    mx.nruns = (int)L.runs.size();
    mx.maxnf = L.maxnf;
    mx.params = L.dparams.as<double>();
    mx.dxinv = L.ddxinv.as<double>();
    mx.f32 = L.precision == kF32;
    mx.stream = stream;
    for (int s = 0; s < 6; s++) {
        mx.step = s;
        launch_maxwell(mx);
    }
    kernel_launches += 18;
    VX_CUDA(cudaGetLastError());
}

void Engine::moments_only(const std::vector<Run *> &set) {
    LaunchSet &L = get_set(set);
    MomLaunch ml{};
    ml.patches = L.dpatch.p;
    ml.colpatch = L.dcolpatch.as<int>();
    ml.colidx = L.dcolidx.as<int>();
    ml.ncols = L.ncols;
    ml.maxnp = L.maxnp;
    ml.fields = L.dfields.as<RunFields>();
    ml.nruns = (int)L.runs.size();
    ml.maxnf = L.maxnf;
    ml.fast = L.precision == kF64 ? L.fast64 : 0;
    ml.stream = stream;
    run_moments(L, ml);
    AsmLaunch al{};
    al.patches = L.dpatch.p;
    al.lvl_ptr = L.dlvl_ptr.as<int>();
    al.lvl_off = L.dlvl_off.as<int>();
    al.lvl_patch = L.dlvl_patch.as<int>();
    al.run_n = L.drun_n.as<int>();
    al.run_ns = L.drun_ns.as<int>();
    al.run_nl = L.drun_nl.as<int>();
    al.nruns = (int)L.runs.size();
    al.maxn = L.maxn;
    al.pairs = L.precision == kF32 ? 1 : 0;
    al.fields = L.dfields.as<RunFields>();
    al.stream = stream;
    launch_assemble(al);
    kernel_launches += 3;
}

}  // namespace vx
