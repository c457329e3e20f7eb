// User problems given as C callbacks (vx_run_create_hooks) and the per-class stage calls
// (vx_run_moments, vx_run_poisson, vx_run_vlasov_stage, vx_run_update_time,
// vx_run_maxwell_stage, vx_run_flag).
//
// The reference's user writes veritas.cpp — initialConditions, Settings::settingsOverride,
// InitialDistribution, GetBY/GetBZ, RefinementOverride (veritas.cpp:7-115) — and
// recompiles.  CallbackProblem is a vx::Problem whose hooks forward to the C callbacks,
// exchanging the reference's structs (Settings.hpp:4-65) as their C mirrors in vx.h.
#include <cstring>
#include <string>

#include "capi_internal.hpp"

namespace vx {
namespace {

template <class V>
void put_vec(const V &v, int32_t *n, double *out, int cap, const char *what) {
    if ((int)v.size() > cap) throw std::invalid_argument(std::string(what) + " has more than " + std::to_string(cap) + " entries");
    *n = (int32_t)v.size();
    for (size_t i = 0; i < v.size(); i++) out[i] = v[i];
}

std::vector<double> get_vec(int32_t n, const double *in, int cap, const char *what) {
    if (n < 0 || n > cap) throw std::invalid_argument(std::string(what) + ": bad entry count " + std::to_string(n));
    return std::vector<double>(in, in + n);
}

// Input / Particles / Output <-> their C mirrors.
void to_c(const Input &g, vx_input &c) {
    std::memset(&c, 0, sizeof c);
    c.minEfficiency = g.minEfficiency;
    c.dx = g.dx;
    c.k = g.k;
    c.refinementCriteria = g.refinementCriteria;
    c.cfl = g.cfl;
    c.sizeWeight = g.sizeWeight;
    c.preLength = g.preLength;
    c.postLength = g.postLength;
    c.nx = g.nx;
    c.r = g.r;
    c.Lfinest = g.Lfinest;
    c.plasma_xl_bound = g.plasma_xl_bound;
    c.plasma_xr_bound = g.plasma_xr_bound;
    put_vec(g.tempEM, &c.ntempEM, c.tempEM, VX_MAX_MISC, "tempEM");
}
void from_c(const vx_input &c, Input &g) {
    g.minEfficiency = c.minEfficiency;
    g.dx = c.dx;
    g.k = c.k;
    g.refinementCriteria = c.refinementCriteria;
    g.cfl = c.cfl;
    g.sizeWeight = c.sizeWeight;
    g.preLength = c.preLength;
    g.postLength = c.postLength;
    g.nx = c.nx;
    g.r = c.r;
    g.Lfinest = c.Lfinest;
    g.plasma_xl_bound = c.plasma_xl_bound;
    g.plasma_xr_bound = c.plasma_xr_bound;
    g.tempEM = get_vec(c.ntempEM, c.tempEM, VX_MAX_MISC, "tempEM");
}
void to_c(const Particles &p, vx_particles &c) {
    std::memset(&c, 0, sizeof c);
    const size_t ns = p.mass.size();
    if (ns > VX_MAX_SPECIES || p.charge.size() != ns || p.np.size() != ns || p.dp.size() != ns ||
        p.pmin.size() != ns || p.misc.size() != ns)
        throw std::invalid_argument("Particles: inconsistent species vectors");
    c.nspecies = (int32_t)ns;
    for (size_t s = 0; s < ns; s++) {
        c.mass[s] = p.mass[s];
        c.charge[s] = p.charge[s];
        c.np[s] = p.np[s];
        c.dp[s] = p.dp[s];
        c.pmin[s] = p.pmin[s];
        put_vec(p.misc[s], &c.nmisc[s], c.misc[s], VX_MAX_MISC, "misc");
    }
}
void from_c(const vx_particles &c, Particles &p) {
    if (c.nspecies < 1 || c.nspecies > VX_MAX_SPECIES)
        throw std::invalid_argument("Particles: nspecies must be in 1.." + std::to_string(VX_MAX_SPECIES));
    p.mass.clear(), p.charge.clear(), p.np.clear(), p.dp.clear(), p.pmin.clear(), p.misc.clear();
    for (int s = 0; s < c.nspecies; s++) {
        p.mass.push_back(c.mass[s]);
        p.charge.push_back(c.charge[s]);
        p.np.push_back(c.np[s]);
        p.dp.push_back(c.dp[s]);
        p.pmin.push_back(c.pmin[s]);
        p.misc.push_back(get_vec(c.nmisc[s], c.misc[s], VX_MAX_MISC, "misc"));
    }
}
void to_c(const Output &o, vx_output &c) {
    c.time = o.time, c.rectangleData = o.rectangleData, c.charge = o.charge, c.energy = o.energy;
    c.potential = o.potential, c.EFieldLongitudinal = o.EFieldLongitudinal;
    c.EFieldTransverse = o.EFieldTransverse, c.BFieldTransverse = o.BFieldTransverse;
    c.AFieldSquared = o.AFieldSquared, c.precision = o.precision;
}
void from_c(const vx_output &c, Output &o) {
    o.time = c.time != 0, o.rectangleData = c.rectangleData != 0, o.charge = c.charge != 0;
    o.energy = c.energy != 0, o.potential = c.potential != 0, o.EFieldLongitudinal = c.EFieldLongitudinal != 0;
    o.EFieldTransverse = c.EFieldTransverse != 0, o.BFieldTransverse = c.BFieldTransverse != 0;
    o.AFieldSquared = c.AFieldSquared != 0, o.precision = c.precision;
}

// Settings -> its C view (what the hooks read).
void to_c(const Settings &s, vx_settings &c) {
    std::memset(&c, 0, sizeof c);
    c.dx = s.dx, c.time = s.time, c.minEfficiency = s.minEfficiency, c.preLength = s.preLength;
    c.postLength = s.postLength, c.refinementCriteria = s.refinementCriteria, c.cfl = s.cfl;
    c.sizeWeight = s.sizeWeight, c.plasma_xl_bound = s.plasma_xl_bound, c.plasma_xr_bound = s.plasma_xr_bound;
    const size_t ns = s.m.size();
    if (ns > VX_MAX_SPECIES) throw std::invalid_argument("too many species");
    c.nspecies = (int32_t)ns;
    for (size_t i = 0; i < ns; i++) {
        c.m[i] = s.m[i];
        c.q[i] = s.q[i];
        c.m_inv[i] = i < s.m_inv.size() ? s.m_inv[i] : 0.0;
        c.dp[i] = s.dp[i];
        c.fMax[i] = i < s.fMax.size() ? s.fMax[i] : 0.0;
        c.pmin[i] = s.pmin[i];
        put_vec(s.temp[i], &c.ntemp[i], c.temp[i], VX_MAX_MISC, "temp");
        c.p_size[i] = s.p_size[i];
        c.p_size_finest[i] = i < s.p_size_finest.size() ? s.p_size_finest[i] : 0;
    }
    put_vec(s.tempEM, &c.ntempEM, c.tempEM, VX_MAX_MISC, "tempEM");
    c.x_size_finest = s.x_size_finest, c.x_size = s.x_size, c.refinementRatio = s.refinementRatio;
    c.maxDepth = s.maxDepth, c.quadratureDepth = s.quadratureDepth;
}
// What settingsOverride may assign back (the derived members are recomputed after it).
void from_c(const vx_settings &c, Settings &s) {
    if (c.nspecies != (int32_t)s.m.size()) throw std::invalid_argument("settings_override may not change nspecies");
    s.dx = c.dx, s.time = c.time, s.minEfficiency = c.minEfficiency, s.preLength = c.preLength;
    s.postLength = c.postLength, s.refinementCriteria = c.refinementCriteria, s.cfl = c.cfl;
    s.sizeWeight = c.sizeWeight, s.plasma_xl_bound = c.plasma_xl_bound, s.plasma_xr_bound = c.plasma_xr_bound;
    for (int i = 0; i < c.nspecies; i++) {
        s.m[i] = c.m[i];
        s.q[i] = c.q[i];
        s.dp[i] = c.dp[i];
        s.pmin[i] = c.pmin[i];
        s.temp[i] = get_vec(c.ntemp[i], c.temp[i], VX_MAX_MISC, "temp");
        s.p_size[i] = c.p_size[i];
    }
    s.tempEM = get_vec(c.ntempEM, c.tempEM, VX_MAX_MISC, "tempEM");
    s.x_size = c.x_size, s.refinementRatio = c.refinementRatio;
    s.maxDepth = c.maxDepth, s.quadratureDepth = c.quadratureDepth;
}

class CallbackProblem : public Problem {
public:
    explicit CallbackProblem(const vx_hooks &h) : H(h) { std::memset(&view, 0, sizeof view); }
    void initialConditions(Input &grid, Particles &particles, Output &output) override {
        vx_input g;
        vx_particles p;
        vx_output o;
        to_c(grid, g);
        to_c(particles, p);
        to_c(output, o);
        H.initial_conditions(H.user, &g, &p, &o);
        from_c(g, grid);
        from_c(p, particles);
        from_c(o, output);
    }
    void settingsOverride(Settings &s) override {
        to_c(s, view);
        if (H.settings_override) {
            H.settings_override(H.user, &view);
            from_c(view, s);
            to_c(s, view);
        }
    }
    void settingsComplete(const Settings &s) override { to_c(s, view); }
    double InitialDistribution(const Settings &, double x, double p, int sp) const override {
        return H.initial_distribution(H.user, &view, x, p, sp);
    }
    double GetBY(const Settings &, double x, double t) const override {
        return H.get_by ? H.get_by(H.user, &view, x, t) : 0.0;
    }
    double GetBZ(const Settings &, double x, double t) const override {
        return H.get_bz ? H.get_bz(H.user, &view, x, t) : 0.0;
    }
    bool RefinementOverride(const Settings &, double x, double p, int depth, int sp) const override {
        return H.refinement_override ? H.refinement_override(H.user, &view, x, p, depth, sp) != 0 : false;
    }
    bool HasRefinementOverride() const override { return H.refinement_override != nullptr; }
    vx_hooks H;
    vx_settings view;
};

}  // namespace
}  // namespace vx

using vx::guard;

extern "C" {

void vx_input_defaults(vx_input *grid, vx_particles *particles, vx_output *output) {
    if (grid) vx::to_c(vx::Input(), *grid);
    if (particles) vx::to_c(vx::Particles(), *particles);
    if (output) vx::to_c(vx::Output(), *output);
}

int vx_run_create_hooks(vx_ctx *ctx, const vx_hooks *hooks, int precision, int poisson, vx_run **out) {
    if (!ctx || !hooks || !out) return VX_ERR_INVALID;
    return guard([&] {
        if (!hooks->initial_conditions || !hooks->initial_distribution)
            throw std::invalid_argument("hooks: initial_conditions and initial_distribution are required");
        if (precision != 64 && precision != 32) throw std::invalid_argument("precision must be 64 or 32");
        if (poisson != vx::kPoissonLU && poisson != vx::kPoissonScan)
            throw std::invalid_argument("poisson must be 0 (LU) or 1 (scan)");
        auto r = std::make_unique<vx_run>();
        r->ctx = ctx;
        r->run.reset(new vx::Run(*ctx->eng, std::make_shared<vx::CallbackProblem>(*hooks), precision));
        r->run->poisson = poisson;
        r->run->init();
        ctx->eng->runs.push_back(r->run.get());
        *out = r.release();
    });
}

int vx_run_settings(vx_run *run, vx_settings *out) {
    if (!run || !out) return VX_ERR_INVALID;
    return guard([&] { vx::to_c(*run->run->S, *out); });
}

int vx_run_moments(vx_run *run) {
    if (!run) return VX_ERR_INVALID;
    return guard([&] { run->ctx->eng->run_phases(*run->run, 0, 0.0, vx::kPhMoments); });
}

int vx_run_poisson(vx_run *run) {
    if (!run) return VX_ERR_INVALID;
    return guard([&] { run->ctx->eng->run_phases(*run->run, 0, 0.0, vx::kPhPoisson); });
}

int vx_run_vlasov_stage(vx_run *run, int stage, double dt, unsigned sub_mask) {
    if (!run || stage < 0 || stage > 5 || !(dt >= 0) || (sub_mask & ~0xfu)) return VX_ERR_INVALID;
    return guard([&] {
        unsigned ph = 0;
        if (sub_mask & VX_SUB_FLUX) ph |= vx::kPhSub0;
        if (sub_mask & VX_SUB_LIMIT) ph |= vx::kPhSub1;
        if (sub_mask & VX_SUB_UPDATE) ph |= vx::kPhSub2;
        if (sub_mask & VX_SUB_COPY) ph |= vx::kPhSub3;
        run->ctx->eng->run_phases(*run->run, stage, dt, ph);
    });
}

int vx_run_update_time(vx_run *run, int stage, double dt) {
    if (!run || stage < 0 || stage > 5 || !(dt >= 0)) return VX_ERR_INVALID;
    return guard([&] { run->run->S->UpdateTime(stage, dt); });
}

int vx_run_maxwell_stage(vx_run *run, int stage, double dt) {
    if (!run || stage < 0 || stage > 5 || !(dt >= 0)) return VX_ERR_INVALID;
    return guard([&] { run->ctx->eng->run_phases(*run->run, stage, dt, vx::kPhMaxwell); });
}

int vx_run_flag(vx_run *run, int species, int depth, int32_t *ij_out, int cap, int *count) {
    if (!run || !count || cap < 0 || (cap > 0 && !ij_out)) return VX_ERR_INVALID;
    return guard([&] {
        vx::Run &R = *run->run;
        if (species < 0 || species >= (int)R.rects.size()) throw std::invalid_argument("no such species");
        if (depth < 0 || depth > R.S->maxDepth) throw std::invalid_argument("no such depth");
        auto flags = R.flag_cells();  // per patch of R.flat
        int n = 0;
        for (size_t k = 0; k < R.flat.size(); k++) {
            const vx::Rect &P = *R.flat[k];
            if (P.species != species || P.depth != depth) continue;
            for (auto &c : flags[k]) {
                if (n < cap) {
                    ij_out[2 * n] = c.first;
                    ij_out[2 * n + 1] = c.second;
                }
                n++;
            }
        }
        *count = n;
    });
}

}  // extern "C"
