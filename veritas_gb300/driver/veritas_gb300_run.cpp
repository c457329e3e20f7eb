// Stand-alone driver over the C++ interface (include/veritas_gb300.hpp), shaped like the
// reference's veritas.cpp main loop: create the solve, step with the CFL time step,
// regrid every K steps, dump the final state.
//
//   veritas_gb300_run [key=value ...]
// Problem keys as in vx_problem (L nx np levels r pmax dens x1..x4 Te p0 pert_amp pert_k
// a0 fwhm delay cfl minEff crit sizeWeight quadDepth bdens bp0 bTe precision), plus
// steps=N  regrid_every=K  dump=path  device=D.  Prints one JSON line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

#include "veritas_gb300.hpp"

int main(int argc, char **argv) {
    std::map<std::string, std::string> kv;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto eq = a.find('=');
        if (eq == std::string::npos) {
            std::fprintf(stderr, "bad argument %s (key=value expected)\n", a.c_str());
            return 2;
        }
        kv[a.substr(0, eq)] = a.substr(eq + 1);
    }
    auto d = [&](const char *k, double def) { return kv.count(k) ? std::stod(kv[k]) : def; };
    auto l = [&](const char *k, long long def) { return kv.count(k) ? std::stoll(kv[k]) : def; };
    vx_problem p;
    vx_problem_defaults(&p);
    p.L = d("L", p.L);
    p.nx = (uint32_t)l("nx", p.nx);
    p.np = (uint32_t)l("np", p.np);
    p.Lfinest = (uint32_t)l("levels", p.Lfinest);
    p.r = (uint32_t)l("r", p.r);
    p.pmax = d("pmax", p.pmax);
    p.dens = d("dens", p.dens);
    p.x1 = d("x1", p.x1);
    p.x2 = d("x2", p.x2);
    p.x3 = d("x3", p.x3);
    p.x4 = d("x4", p.x4);
    p.Te = d("Te", p.Te);
    p.p0 = d("p0", p.p0);
    p.pert_amp = d("pert_amp", p.pert_amp);
    p.pert_k = d("pert_k", p.pert_k);
    p.a0 = d("a0", p.a0);
    p.fwhm = d("fwhm", p.fwhm);
    p.delay = d("delay", p.delay);
    p.cfl = d("cfl", p.cfl);
    p.minEff = d("minEff", p.minEff);
    p.crit = d("crit", p.crit);
    p.sizeWeight = d("sizeWeight", p.sizeWeight);
    p.quadDepth = (int32_t)l("quadDepth", p.quadDepth);
    p.bdens = d("bdens", p.bdens);
    p.bp0 = d("bp0", p.bp0);
    p.bTe = d("bTe", p.bTe);
    p.precision = (int32_t)l("precision", p.precision);
    const long long steps = l("steps", 10), regrid_every = l("regrid_every", 0);
    try {
        veritas_gb300::Context ctx((int)l("device", 0));
        veritas_gb300::SolverManager SM(ctx, p);
        auto t0 = std::chrono::steady_clock::now();
        for (long long s = 1; s <= steps; s++) {
            SM.Advance(SM.CalculateDt(p.cfl));
            if (regrid_every > 0 && s % regrid_every == 0) SM.reGrid(SM.time());
        }
        ctx.sync();
        double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (kv.count("dump")) SM.saveState(kv["dump"]);
        std::printf("{\"steps\": %lld, \"time\": %.17g, \"cells\": %lld, \"seconds\": %.6f}\n", steps, SM.time(),
                    SM.cells(), secs);
    } catch (const veritas_gb300::Error &e) {
        std::fprintf(stderr, "error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
