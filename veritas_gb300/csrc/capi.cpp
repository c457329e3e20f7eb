// extern "C" entry points declared in include/vx.h.
#include <cstring>
#include <string>

#include "capi_internal.hpp"

using vx::guard;

namespace {
vx::LaserSlabParams to_params(const vx_problem &p) {
    vx::LaserSlabParams q;
    q.lambda = p.lambda;
    q.L = p.L;
    q.nx = p.nx;
    q.np = p.np;
    q.Lfinest = p.Lfinest;
    q.r = p.r;
    q.pmax = p.pmax;
    q.dens = p.dens;
    q.x1 = p.x1;
    q.x2 = p.x2;
    q.x3 = p.x3;
    q.x4 = p.x4;
    q.Te = p.Te;
    q.p0 = p.p0;
    q.pert_amp = p.pert_amp;
    q.pert_k = p.pert_k;
    q.a0 = p.a0;
    q.fwhm = p.fwhm;
    q.delay = p.delay;
    q.cfl = p.cfl;
    q.minEff = p.minEff;
    q.crit = p.crit;
    q.sizeWeight = p.sizeWeight;
    q.quadDepth = p.quadDepth;
    q.bdens = p.bdens;
    q.bp0 = p.bp0;
    q.bTe = p.bTe;
    q.mi = p.mi;
    q.iTe = p.iTe;
    q.ipmax = p.ipmax;
    return q;
}

std::unique_ptr<vx::Settings> host_settings(const vx_problem &p) {
    auto prob = std::make_shared<vx::LaserSlab>(to_params(p));
    vx::Input grid;
    vx::Particles particles;
    vx::Output output;
    prob->initialConditions(grid, particles, output);
    return std::unique_ptr<vx::Settings>(new vx::Settings(grid, particles, output, prob));
}
}  // namespace

namespace vx {
thread_local std::string g_err;
// Error message for entry points defined outside this file.
void set_last_error(const std::string &msg) { g_err = msg; }
}  // namespace vx


extern "C" {

void vx_problem_defaults(vx_problem *p) {
    vx::LaserSlabParams d;
    std::memset(p, 0, sizeof *p);
    p->lambda = d.lambda;
    p->L = d.L;
    p->nx = d.nx;
    p->np = d.np;
    p->Lfinest = d.Lfinest;
    p->r = d.r;
    p->pmax = d.pmax;
    p->dens = d.dens;
    p->x1 = d.x1;
    p->x2 = d.x2;
    p->x3 = d.x3;
    p->x4 = d.x4;
    p->Te = d.Te;
    p->p0 = d.p0;
    p->pert_amp = d.pert_amp;
    p->pert_k = d.pert_k;
    p->a0 = d.a0;
    p->fwhm = d.fwhm;
    p->delay = d.delay;
    p->cfl = d.cfl;
    p->minEff = d.minEff;
    p->crit = d.crit;
    p->sizeWeight = d.sizeWeight;
    p->quadDepth = d.quadDepth;
    p->precision = 64;
    p->bdens = d.bdens;
    p->bp0 = d.bp0;
    p->bTe = d.bTe;
    p->poisson = 0;
    p->fast = 0;
    p->mi = d.mi;
    p->iTe = d.iTe;
    p->ipmax = d.ipmax;
}

const char *vx_last_error(void) { return vx::g_err.c_str(); }

int vx_ctx_create(int device, vx_ctx **out) {
    if (!out) return VX_ERR_INVALID;
    return guard([&] {
        auto c = new vx_ctx;
        try {
            c->eng.reset(new vx::Engine(device));
        } catch (...) {
            delete c;
            throw;
        }
        *out = c;
    });
}

int vx_ctx_destroy(vx_ctx *ctx) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] {
        if (!ctx->eng->runs.empty())
            throw std::invalid_argument("context still has " + std::to_string(ctx->eng->runs.size()) +
                                        " run(s): destroy them first");
        delete ctx;
    });
}

int vx_ctx_sync(vx_ctx *ctx) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->sync(); });
}

int vx_ctx_set_launch_mode(vx_ctx *ctx, int graphs, int pdl) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->set_launch_mode(graphs != 0, pdl != 0); });
}

int vx_ctx_set_persistent(vx_ctx *ctx, int on) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->set_persistent(on != 0); });
}

int vx_ctx_set_persistent_limit(vx_ctx *ctx, uint64_t limit_ns, int phantom) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->set_persistent_limit(limit_ns, phantom); });
}

int vx_ctx_set_pipelined(vx_ctx *ctx, int on) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->set_pipelined(on != 0); });
}

int vx_ctx_kernel_launches(vx_ctx *ctx, uint64_t *out) {
    if (!ctx || !out) return VX_ERR_INVALID;
    *out = ctx->eng->kernel_launches;
    return VX_OK;
}

int vx_run_create(vx_ctx *ctx, const vx_problem *prob, vx_run **out) {
    if (!ctx || !prob || !out) return VX_ERR_INVALID;
    return guard([&] {
        if (prob->precision != 64 && prob->precision != 32) throw std::invalid_argument("precision must be 64 or 32");
        auto r = std::make_unique<vx_run>();
        r->ctx = ctx;
        if (prob->poisson != vx::kPoissonLU && prob->poisson != vx::kPoissonScan)
            throw std::invalid_argument("poisson must be 0 (LU) or 1 (scan)");
        if (prob->fast != 0 && prob->fast != 1) throw std::invalid_argument("fast must be 0 or 1");
        r->run.reset(new vx::Run(*ctx->eng, std::make_shared<vx::LaserSlab>(to_params(*prob)), prob->precision));
        r->run->poisson = prob->poisson;
        r->run->fast64 = prob->precision == 64 ? prob->fast : 0;
        r->run->init();
        ctx->eng->runs.push_back(r->run.get());
        *out = r.release();
    });
}

int vx_run_destroy(vx_run *run) {
    if (!run) return VX_ERR_INVALID;
    return guard([&] {
        run->ctx->eng->sync();
        delete run;
    });
}

int vx_run_calculate_dt(vx_run *run, double *dt) {
    if (!run || !dt) return VX_ERR_INVALID;
    return guard([&] { *dt = run->run->calculate_dt(); });
}

int vx_run_advance(vx_run *run, double dt) {
    if (!run || !(dt >= 0)) return VX_ERR_INVALID;
    return guard([&] { run->run->advance(dt); });
}

int vx_run_advance_fields(vx_run *run, double dt) {
    if (!run || !(dt >= 0)) return VX_ERR_INVALID;
    return guard([&] { run->run->advance_fields(dt); });
}

int vx_run_regrid(vx_run *run) {
    if (!run) return VX_ERR_INVALID;
    return guard([&] { run->run->regrid(false); });
}

int vx_run_layout(vx_run *run, int32_t *out, int cap, int *count) {
    if (!run || !count || cap < 0 || (cap > 0 && !out)) return VX_ERR_INVALID;
    return guard([&] {
        int k = 0;
        for (auto &sp : run->run->rects)
            for (auto &lvl : sp)
                for (auto &r : lvl) {
                    if (k < cap) {
                        int32_t *o = out + 6 * k;
                        o[0] = r->species;
                        o[1] = r->depth;
                        o[2] = r->x_pos;
                        o[3] = r->p_pos;
                        o[4] = r->n_x;
                        o[5] = r->n_p;
                    }
                    k++;
                }
        *count = k;
    });
}

int vx_error_weights(const vx_problem *prob, int species, int depth, double *w5, double *crit) {
    if (!prob || !w5 || !crit) return VX_ERR_INVALID;
    return guard([&] {
        auto S = host_settings(*prob);
        if (species < 0 || species >= (int)S->q.size() || depth < 0 || depth > S->maxDepth)
            throw std::invalid_argument("species or depth out of range");
        vx::error_weights(*S, depth, species, w5);
        *crit = S->refinementCriteria;
    });
}

int vx_update_hierarchy(const vx_problem *prob, int species, const int32_t *patches, int npatches,
                        const int32_t *flag_ptr, const int32_t *flag_ij, int32_t *out, int cap, int *count) {
    if (!prob || !patches || npatches <= 0 || !flag_ptr || !count || cap < 0 || (cap > 0 && !out))
        return VX_ERR_INVALID;
    return guard([&] {
        auto S = host_settings(*prob);
        const vx::Settings &s = *S;
        if (species < 0 || species >= (int)s.q.size()) throw std::invalid_argument("species out of range");
        std::vector<vx::Run::BoxList> H;
        std::vector<std::vector<int>> at_depth(s.maxDepth + 1);
        for (int k = 0; k < npatches; k++) {
            const int32_t *r = patches + 5 * k;
            if (r[0] < 0 || r[0] > s.maxDepth) throw std::invalid_argument("patch depth out of range");
            if (flag_ptr[k + 1] < flag_ptr[k]) throw std::invalid_argument("flag_ptr must not decrease");
            at_depth[r[0]].push_back(k);
        }
        if (flag_ptr[0] != 0 || (flag_ptr[npatches] > 0 && !flag_ij)) throw std::invalid_argument("bad flag list");
        for (int d = s.maxDepth; d >= 0 && !at_depth[d].empty(); d--) {
            vx::Run::BoxList b;
            for (int k : at_depth[d]) {
                const int32_t *r = patches + 5 * k;
                b.push_back({{r[1], r[2]}, {r[1] + r[3], r[2] + r[4]}});
            }
            H.push_back(b);
        }
        if (H.empty()) throw std::invalid_argument("no base-level patch");
        auto level_flags = [&](int l) {
            std::vector<std::pair<int, int>> f;
            for (int k : at_depth[s.maxDepth - l])
                for (int q = flag_ptr[k]; q < flag_ptr[k + 1]; q++) f.push_back({flag_ij[2 * q], flag_ij[2 * q + 1]});
            return f;
        };
        auto geo = vx::promote_geometry(s, species, vx::update_hierarchy(s, species, H, level_flags));
        for (size_t k = 0; k < geo.size() && (int)k < cap; k++) {
            int32_t *o = out + 9 * k;
            const vx::PatchGeom &g = geo[k];
            o[0] = g.depth;
            o[1] = g.x_pos;
            o[2] = g.p_pos;
            o[3] = g.n_x;
            o[4] = g.n_p;
            o[5] = g.up;
            o[6] = g.down;
            o[7] = g.left;
            o[8] = g.right;
        }
        *count = (int)geo.size();
    });
}

int vx_runs_calculate_dt(vx_run *const *runs, double *dt, int nruns) {
    if (!runs || !dt || nruns <= 0) return VX_ERR_INVALID;
    return guard([&] {
        std::vector<vx::Run *> set;
        vx_ctx *c = runs[0]->ctx;
        for (int i = 0; i < nruns; i++) {
            if (!runs[i] || runs[i]->ctx != c) throw std::invalid_argument("runs must belong to one context");
            set.push_back(runs[i]->run.get());
        }
        auto v = c->eng->calculate_dt(set);
        for (int i = 0; i < nruns; i++) dt[i] = v[i];
    });
}

int vx_runs_autotune(vx_run *const *runs, int nruns, int *tile_j, int *tile_i) {
    if (!runs || nruns <= 0) return VX_ERR_INVALID;
    return guard([&] {
        std::vector<vx::Run *> set;
        vx_ctx *c = runs[0]->ctx;
        for (int i = 0; i < nruns; i++) {
            if (!runs[i] || runs[i]->ctx != c) throw std::invalid_argument("runs must belong to one context");
            set.push_back(runs[i]->run.get());
        }
        auto best = c->eng->autotune(set, 5);
        if (tile_j) *tile_j = best.first;
        if (tile_i) *tile_i = best.second;
    });
}

int vx_runs_advance(vx_run *const *runs, const double *dt, int nruns) {
    if (!runs || !dt || nruns <= 0) return VX_ERR_INVALID;
    return guard([&] {
        std::vector<vx::Run *> set;
        std::vector<double> d;
        vx_ctx *c = runs[0]->ctx;
        for (int i = 0; i < nruns; i++) {
            if (!runs[i] || runs[i]->ctx != c) throw std::invalid_argument("runs must belong to one context");
            set.push_back(runs[i]->run.get());
            d.push_back(dt[i]);
        }
        c->eng->advance(set, d);
    });
}

int vx_run_time(vx_run *run, double *t) {
    if (!run || !t) return VX_ERR_INVALID;
    *t = run->run->S->time;
    return VX_OK;
}

int vx_run_cell_count(vx_run *run, int64_t *cells) {
    if (!run || !cells) return VX_ERR_INVALID;
    *cells = run->run->cell_count();
    return VX_OK;
}

int vx_run_load_state(vx_run *run, const char *path) {
    if (!run || !path) return VX_ERR_INVALID;
    int rc = guard([&] { run->run->load_state(path); });
    return (rc == VX_ERR_STATE) ? VX_ERR_IO : rc;
}

int vx_run_save_state(vx_run *run, const char *path) {
    if (!run || !path) return VX_ERR_INVALID;
    int rc = guard([&] { run->run->save_state(path); });
    return (rc == VX_ERR_STATE) ? VX_ERR_IO : rc;
}

int vx_run_write_fields(vx_run *run, const char *dir, uint32_t mask, int digits, double t) {
    if (!run || !dir || digits < 0 || digits > 40 || (mask & ~(uint32_t)VX_OUT_ALL)) return VX_ERR_INVALID;
    int rc = guard([&] { run->run->write_fields(dir, mask, digits, t); });
    return (rc == VX_ERR_STATE) ? VX_ERR_IO : rc;
}

int vx_run_write_rectangles(vx_run *run, const char *dir, double t) {
    if (!run || !dir) return VX_ERR_INVALID;
    int rc = guard([&] { run->run->write_rectangles(dir, t); });
    return (rc == VX_ERR_STATE) ? VX_ERR_IO : rc;
}

int vx_run_get_field(vx_run *run, int which, double *out, int64_t *len) {
    if (!run || !len) return VX_ERR_INVALID;
    return guard([&] {
        vx::Run &R = *run->run;
        const double *src = nullptr;
        int64_t n = 0;
        switch (which) {
            case 0: src = R.F.By; n = R.nf; break;
            case 1: src = R.F.Bz; n = R.nf; break;
            case 2: src = R.F.Ey; n = R.nf; break;
            case 3: src = R.F.Ez; n = R.nf; break;
            case 4: src = R.F.Ay; n = R.nf; break;
            case 5: src = R.F.Az; n = R.nf; break;
            case 6: src = R.F.asq; n = R.n + 1; break;
            case 7: src = R.F.phi; n = R.n; break;
            case 8: src = R.F.charge; n = R.n; break;
            case 9: src = R.F.J; n = R.n; break;
            case 10: src = R.F.efin; n = R.n; break;
            default: throw std::invalid_argument("unknown field id");
        }
        *len = n;
        if (out) {
            R.eng->sync();
            VX_CUDA(cudaMemcpy(out, src, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
        }
    });
}

int vx_ctx_timer_begin(vx_ctx *ctx) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->timer_begin(); });
}

int vx_ctx_timer_end(vx_ctx *ctx, double *ms) {
    if (!ctx || !ms) return VX_ERR_INVALID;
    return guard([&] { *ms = ctx->eng->timer_end(); });
}

int vx_run_profile_kernels(vx_run *run, int reps, double *out_ms, int cap, int *count) {
    if (!run || !out_ms || !count || reps <= 0 || cap <= 0) return VX_ERR_INVALID;
    return guard([&] {
        auto v = run->ctx->eng->profile_kernels(*run->run, reps);
        int k = 0;
        for (; k < (int)v.size() && k < cap; k++) out_ms[k] = v[k];
        *count = k;
    });
}

int vx_ctx_flush_l2(vx_ctx *ctx) {
    if (!ctx) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->flush_l2(); });
}

int vx_ctx_measure_fp64_latency(vx_ctx *ctx, double *mul_sub_cycles, double *shfl_cycles) {
    if (!ctx || !mul_sub_cycles || !shfl_cycles) return VX_ERR_INVALID;
    return guard([&] { ctx->eng->measure_fp64_latency(mul_sub_cycles, shfl_cycles); });
}

int vx_ctx_measure_fp64_peak(vx_ctx *ctx, double *gflops) {
    if (!ctx || !gflops) return VX_ERR_INVALID;
    return guard([&] { *gflops = ctx->eng->measure_fp64_peak(); });
}

int vx_host_alloc(size_t bytes, void **out) {
    if (!out || bytes == 0) return VX_ERR_INVALID;
    return guard([&] { VX_CUDA(cudaMallocHost(out, bytes)); });
}

int vx_host_free(void *p) {
    if (!p) return VX_ERR_INVALID;
    return guard([&] { VX_CUDA(cudaFreeHost(p)); });
}

int vx_run_state_size(vx_run *run, int64_t *len) {
    if (!run || !len) return VX_ERR_INVALID;
    return guard([&] { *len = run->run->state_size(); });
}

int vx_run_state_to_host(vx_run *run, double *state_out) {
    if (!run || !state_out) return VX_ERR_INVALID;
    return guard([&] { run->run->state_to_host(state_out); });
}

int vx_run_step_host(vx_run *run, const double *state_in, double *state_out, double dt) {
    if (!run || !state_in || !state_out || !(dt >= 0)) return VX_ERR_INVALID;
    return guard([&] { run->run->step_host(state_in, state_out, dt); });
}

int vx_server_create(vx_ctx *ctx, uint64_t hbm_budget_bytes, int max_live, vx_server **out) {
    if (!ctx || !out || hbm_budget_bytes == 0 || max_live <= 0) return VX_ERR_INVALID;
    return guard([&] {
        auto s = std::make_unique<vx_server>();
        s->ctx = ctx;
        s->srv.reset(new vx::Server(*ctx->eng, (size_t)hbm_budget_bytes, max_live));
        *out = s.release();
    });
}

int vx_server_destroy(vx_server *s) {
    if (!s) return VX_ERR_INVALID;
    return guard([&] {
        s->ctx->eng->sync();
        delete s;
    });
}

int vx_server_clock(vx_server *s, double *now) {
    if (!s || !now) return VX_ERR_INVALID;
    *now = s->srv->clock();
    return VX_OK;
}

int vx_server_submit(vx_server *s, const vx_problem *p, int64_t steps, double arrival, const char *state_path,
                     int64_t *id) {
    if (!s || !p || !id) return VX_ERR_INVALID;
    return guard([&] {
        *id = s->srv->submit(to_params(*p), p->precision, steps, arrival, state_path ? state_path : "", p->poisson, 1,
                             p->precision == 64 ? p->fast : 0);
    });
}

int vx_server_step(vx_server *s, int *live, int *waiting) {
    if (!s) return VX_ERR_INVALID;
    return guard([&] {
        int l = s->srv->step(s->srv->clock());
        if (live) *live = l;
        if (waiting) *waiting = s->srv->waiting();
    });
}

int vx_server_result(vx_server *s, int64_t id, vx_request_result *out) {
    if (!s || !out) return VX_ERR_INVALID;
    return guard([&] {
        const auto &r = s->srv->request(id);
        std::memset(out, 0, sizeof *out);
        const bool over = r.status == vx::Server::kDone || r.status == vx::Server::kCancelled ||
                          r.status == vx::Server::kFailed;
        out->finished = over ? 1 : 0;
        out->steps_done = r.done_steps;
        out->arrival = r.arrival;
        out->admitted = r.admitted;
        out->finish = r.finish;
        out->sim_time = r.sim_time;
        out->cells = r.cells;
        out->device_bytes = r.bytes;
        out->status = (int32_t)r.status;
        out->regrids = r.regrids;
        out->bound = r.bound;
        std::strncpy(out->error, r.error.c_str(), sizeof out->error - 1);
    });
}

int vx_server_cancel(vx_server *s, int64_t id) {
    if (!s) return VX_ERR_INVALID;
    return guard([&] { s->srv->cancel(id); });
}

int vx_server_set_regrid(vx_server *s, int enable, double after_s) {
    if (!s || !(after_s >= 0)) return VX_ERR_INVALID;
    s->srv->regrid_enabled = enable != 0;
    s->srv->regrid_after = after_s;
    return VX_OK;
}

}  // extern "C"
