// Serving loop: continuous batching of independent solves on one context.
//
// Requests queue in arrival order.  Each call of step() first admits, in order, every
// waiting request whose device-memory estimate fits in what the budget has left (the
// estimate is replaced by the run's real footprint once it exists), then advances every
// live solve by one full RK step in one batched launch set (one launch per sub-step for
// all of them), and retires the solves that reached their step count: their final
// state is written where the request asked and their memory is released before the
// next admission.  A request that arrives while others run joins at the next step;
// nothing waits for the batch to drain.
#include <algorithm>
#include <cmath>

#include "serve.hpp"

namespace vx {

size_t Run::device_bytes() const {
    size_t b = 0;
    for (auto &sp : rects)
        for (auto &lvl : sp)
            for (auto &r : lvl) b += r->slab.bytes + r->cols.bytes + r->masks.bytes;
    for (const DevBuf *d : {&dBy, &dBz, &dEy, &dEz, &dAy, &dAz, &dasq, &dphi, &dcharge, &dJ, &dneut, &defin, &dex0,
                            &dasq32, &defin32, &dacell32, &drelc32, &dlu_perm, &dlb_band, &dlb_fptr, &dlb_fcol, &dlb_fval, &dlb_slot,
                            &dlb_sload, &dlb_take, &dub_band, &dub_diag, &dub_rdiag, &dub_rdlo, &dub_fptr, &dub_fcol,
                            &dub_fval, &dpf_Y, &drelc, &drefc, &dghost_ops, &diface_ops, &dcsync_ops})
        b += d->bytes;
    return b;
}

// Device bytes a request will take: the base level's patch planes times a refinement
// allowance (each further level may cover the base once more at most in cells), plus
// the field arrays and the Poisson operator.
size_t Server::estimate_bytes(const LaserSlabParams &p, int precision) {
    const double levels = std::max(1u, p.Lfinest);
    const double cells = (double)(p.nx + 4) * (p.np / 8 * 8 + 8 + 4);
    const double esize = precision == kF32 ? 4.0 : 8.0;
    const double planes = precision == kF32 ? 23.0 : 28.0;  // FP32: no gamma / face planes
    const double nfine = p.nx * std::pow((double)p.r, levels - 1);
    const double fields = nfine * (8.0 * 6 + 16) * 8.0 + nfine * 24.0 * (precision == kF32 ? 1.0 : 2.0);
    return (size_t)(cells * planes * esize * levels + fields);
}

Server::Server(Engine &e, size_t budget, int max_live) : eng(e), budget_(budget), max_live_(max_live) {}

Server::~Server() = default;

int64_t Server::submit(const LaserSlabParams &p, int precision, int64_t steps, double arrival,
                       const std::string &state_path, int poisson) {
    if (steps <= 0) throw std::invalid_argument("a request needs at least one step");
    if (precision != kF64 && precision != kF32) throw std::invalid_argument("precision must be 64 or 32");
    if (poisson != kPoissonLU && poisson != kPoissonScan) throw std::invalid_argument("poisson must be 0 or 1");
    Request r;
    r.id = next_id_++;
    r.params = p;
    r.precision = precision;
    r.poisson = precision == kF32 ? kPoissonScan : poisson;
    r.steps = steps;
    r.arrival = arrival;
    r.state_path = state_path;
    r.estimate = estimate_bytes(p, precision);
    if (r.estimate > budget_) throw std::invalid_argument("request larger than the whole memory budget");
    waiting_.push_back(r.id);
    reqs_.emplace(r.id, std::move(r));
    return next_id_ - 1;
}

void Server::admit(double now) {
    while (!waiting_.empty() && (int)live_.size() < max_live_) {
        Request &r = reqs_.at(waiting_.front());
        if (used_ + r.estimate > budget_) break;  // in order: the head blocks the queue
        waiting_.pop_front();
        r.admitted = now;
        r.run.reset(new Run(eng, std::make_shared<LaserSlab>(r.params), r.precision));
        r.run->poisson = r.poisson;
        r.run->init();
        r.bytes = r.run->device_bytes();
        used_ += r.bytes;
        live_.push_back(r.id);
    }
}

int Server::step(double now) {
    admit(now);
    if (live_.empty()) return 0;
    std::vector<Run *> set;
    for (int64_t id : live_) set.push_back(reqs_.at(id).run.get());
    // one launch set per precision and Poisson solver (different kernels); the sets of
    // earlier mixes are dropped, so cached tables do not pile up beside the budget
    std::vector<std::vector<Run *>> used;
    for (int prec : {kF64, kF32})
        for (int pois : {kPoissonLU, kPoissonScan}) {
            std::vector<Run *> part;
            for (Run *r : set)
                if (r->precision == prec && r->poisson == pois) part.push_back(r);
            if (part.empty()) continue;
            auto dt = eng.calculate_dt(part);
            eng.advance(part, dt);
            used.push_back(part);
        }
    eng.retain_sets(used);
    eng.sync();
    std::vector<int64_t> still;
    for (int64_t id : live_) {
        Request &r = reqs_.at(id);
        r.done_steps++;
        if (r.done_steps < r.steps) {
            still.push_back(id);
            continue;
        }
        r.finish = clock();
        r.sim_time = r.run->S->time;
        if (!r.state_path.empty()) r.run->save_state(r.state_path);
        used_ -= r.bytes;
        r.cells = r.run->cell_count();
        r.run.reset();
        r.finished = true;
        finished_order_.push_back(id);
    }
    live_ = still;
    return (int)live_.size();
}

const Server::Request &Server::request(int64_t id) const {
    auto it = reqs_.find(id);
    if (it == reqs_.end()) throw std::invalid_argument("unknown request id");
    return it->second;
}

}  // namespace vx
