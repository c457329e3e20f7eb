// FP64 "plain" Vlasov kernels: the per-patch FCT Runge-Kutta sub-steps of
// Rectangle::FCTTimeStep (Rectangle.cpp:1255-1623).
//
// This translation unit is compiled with --fmad=false: every double-precision
// expression below is evaluated with the same operations, operands and order as the
// reference C++ (separate IEEE multiply and add, IEEE division and square root), so the
// results are bit-identical to a non-FMA x86-64 / -ffp-contract=off build of the
// reference for the same inputs.
//
// Work decomposition: every kernel walks a list of 32(p) x 8(x) tiles that covers the
// padded block of every patch of every run in the launch, so one launch per sub-step
// serves a single patch, all patches of an AMR hierarchy, or a batch of independent runs.
//
// Compiled a second time with -DVX_FP64_FAST and contraction allowed: the FP64 form that
// trades the reference's rounding for fewer FP64 instructions (fused multiply-add, the
// WENO weights as one quotient, and the two quotients of a face value through a
// Newton-refined hardware reciprocal instead of five IEEE divisions).  Its kernels
// live in namespace vx::fast64 and its launcher is launch_fct64_substep_fast.
#include <cuda_runtime.h>
#include "fast64.cuh"
#include "vx_kernels.hpp"

#ifdef VX_FP64_FAST
#define VX_FCT64_NS fast64
#define VX_FCT64_LAUNCH launch_fct64_substep_fast
#else
#define VX_FCT64_NS exact64
#define VX_FCT64_LAUNCH launch_fct64_substep
#endif

namespace vx {
namespace VX_FCT64_NS {

using P64 = PatchT<double>;

// WENO-type upwind face value (Rectangle.cpp:980-1030; identical values to
// Rectangle.cpp:943-977).  f1..f4 are the four cells left-to-right around the face.
__device__ __forceinline__ double weno_face(double f1, double f2, double f3, double f4, bool right) {
    const double c6 = 1.0 / 6;
    const double c43 = 4.0 / 3;
    double fL = c6 * (-f1 + 5 * f2 + 2 * f3);
    double fR = c6 * (2 * f2 + 5 * f3 - f4);
    double AL = f1 - 2 * f2 + f3;
    double BL = f3 - f1;
    double AR = f2 - 2 * f3 + f4;
    double BR = f4 - f2;
    double bL = c43 * (AL * AL) + 0.5 * AL * BL + 0.25 * (BL * BL);
    double bR = c43 * (AR * AR) - 0.5 * AR * BR + 0.25 * (BR * BR);
    const double mm = 1.0e-10;
#ifdef VX_FP64_FAST
    // oL / (oL + oR) with o = 0.5 / (mm + b)^2 is dR^2 / (dL^2 + dR^2), d = mm + b
    const double dL = mm + bL, dR = mm + bR;
    double wL = (dR * dR) * rcp_nr(dL * dL + dR * dR);
    double wR = 1.0 - wL;
#else
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
#endif
    double wL0 = wL * (0.75 + wL * (wL - 0.5));
    double wR0 = wR * (0.75 + wR * (wR - 0.5));
    double pick;
    if (right) pick = (wL0 > wR0) ? wL0 : wR0;
    else pick = (wL0 < wR0) ? wL0 : wR0;
#ifdef VX_FP64_FAST
    double fwl = pick * rcp_nr(wL0 + wR0);
#else
    double fwl = pick / (wL0 + wR0);
#endif
    double fwr = 1 - fwl;
    return fwl * fL + fwr * fR;
}

// Both upwind choices of weno_face at once (the smoothness weights do not depend on the
// velocity): out_right / out_left are weno_face(..., true) / weno_face(..., false), bit
// for bit.
__device__ __forceinline__ void weno_face_both(double f1, double f2, double f3, double f4, double &out_right,
                                               double &out_left) {
    const double c6 = 1.0 / 6;
    const double c43 = 4.0 / 3;
    double fL = c6 * (-f1 + 5 * f2 + 2 * f3);
    double fR = c6 * (2 * f2 + 5 * f3 - f4);
    double AL = f1 - 2 * f2 + f3;
    double BL = f3 - f1;
    double AR = f2 - 2 * f3 + f4;
    double BR = f4 - f2;
    double bL = c43 * (AL * AL) + 0.5 * AL * BL + 0.25 * (BL * BL);
    double bR = c43 * (AR * AR) - 0.5 * AR * BR + 0.25 * (BR * BR);
    const double mm = 1.0e-10;
#ifdef VX_FP64_FAST
    const double dL = mm + bL, dR = mm + bR;
    double wL = (dR * dR) * rcp_nr(dL * dL + dR * dR);
    double wR = 1.0 - wL;
#else
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
#endif
    double wL0 = wL * (0.75 + wL * (wL - 0.5));
    double wR0 = wR * (0.75 + wR * (wR - 0.5));
    const double pr = (wL0 > wR0) ? wL0 : wR0, pl = (wL0 < wR0) ? wL0 : wR0;
#ifdef VX_FP64_FAST
    const double inv = rcp_nr(wL0 + wR0);  // one reciprocal for both choices
    double fwl = pr * inv;
    out_right = fwl * fL + (1 - fwl) * fR;
    fwl = pl * inv;
    out_left = fwl * fL + (1 - fwl) * fR;
#else
    double fwl = pr / (wL0 + wR0);
    out_right = fwl * fL + (1 - fwl) * fR;
    fwl = pl / (wL0 + wR0);
    out_left = fwl * fL + (1 - fwl) * fR;
#endif
}

__device__ __forceinline__ double vmax(double a, double b) { return (a > b) ? a : b; }
__device__ __forceinline__ double vmin(double a, double b) { return (a < b) ? a : b; }
// vmax(0.0, x) and vmin(0.0, x) decided on the bit pattern with integer instructions (the
// FP64 unit is the limiter's bottleneck): x < 0 exactly when the sign bit is set and x is
// neither -0 nor NaN; x > 0 when the sign bit is clear and x is neither +0 nor NaN.
__device__ __forceinline__ double vmax0(double x) {
    const long long b = __double_as_longlong(x);
    const long long m = b & 0x7FFFFFFFFFFFFFFFLL;
    return (b < 0 && m != 0 && m <= 0x7FF0000000000000LL) ? 0.0 : x;
}
__device__ __forceinline__ double vmin0(double x) {
    const long long b = __double_as_longlong(x);
    return (b > 0 && b <= 0x7FF0000000000000LL) ? 0.0 : x;
}
// x > 0.0 (false for zeros and NaN) on the bit pattern
__device__ __forceinline__ bool gt0(double x) {
    const long long b = __double_as_longlong(x);
    return b > 0 && b <= 0x7FF0000000000000LL;
}


// Rectangle::GetEfield (Rectangle.cpp:1055-1067): mean of the finest-grid E_x over the
// rtb finest cells under coarse cell i; finest indices are periodic (EMSolver.cpp:137-154).
__device__ __forceinline__ double patch_efield(const P64 &P, const RunFields &F, int i) {
    int x = P.rtb * (i + P.x_pos);
    double t = 0.0;
    for (int k = 0; k < P.rtb; k++) {
        int y = x + k;
        y = (y > -1) ? y : (y + F.n);
        y = (y < F.n) ? y : (y - F.n);
        t += F.efin[y];
    }
    return t * (1.0 / P.rtb);
}

__device__ __forceinline__ double a_sq_face(const P64 &P, const RunFields &F, int i) {
    int x = P.rtb * (i + P.x_pos);
    x = x < 0 ? 0 : (x > F.n ? F.n : x);
    return F.asq[x];
}

#define VX_TILE_PROLOGUE                                  \
    const TileRef t = tiles[blockIdx.x];                  \
    const P64 &P = patches[t.patch];                      \
    const int i = t.i0 + (int)threadIdx.y;                \
    const int j = t.j0 + (int)threadIdx.x;                \
    if (i > P.nx + 1 || j > P.np + 1) return;             \
    const int pit = P.pitch;                              \
    const int id = pidx(i, j, pit);

// Lorentz factor at every (x-face i, p-face j) node, i in [-1,nx+1], j in [-1,np+1]:
// Rectangle::Gamma (Rectangle.hpp:181) with A^2 at the finest face under x-face i
// (EMSolver::GetASquared, EMSolver.cpp:133) and p_j = Momentum(j) (Rectangle.hpp:86).
__global__ void k64_gamma(const P64 *patches, const TileRef *tiles, const RunFields *fields) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < -1 || j < -1) return;
    const RunFields &F = fields[P.run];
    double as = P.qq * a_sq_face(P, F, i);
    double p = P.pmin + P.dp * (double)(j + P.p_pos);
    P.gam[id] = sqrt(1.0 + ((p * p) + as) * P.g2);
}

// Face velocities and reconstructed face values (Rectangle.cpp:1278-1312).
__global__ void k64_faces(const P64 *patches, const TileRef *tiles, const RunFields *fields, int use_f0, int part) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    const double *f = use_f0 ? P.f0 : P.f1;
    const double *g = P.gam;
    if ((part & 1) && i >= 0 && i <= P.nx && j >= -1 && j <= P.np) {
        double am = P.dp_inv * P.cc * (g[pidx(i, j + 1, pit)] - g[id]);
        P.ex[id] = am;
        P.fx[id] = weno_face(f[pidx(i - 2, j, pit)], f[pidx(i - 1, j, pit)], f[id], f[pidx(i + 1, j, pit)], gt0(am));
    }
    if ((part & 2) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np) {
        const RunFields &F = fields[P.run];
        double Em = P.q * patch_efield(P, F, i);
        double am = Em - P.cc * P.dx_inv * (g[pidx(i + 1, j, pit)] - g[id]);
        P.ep[id] = am;
        P.fp[id] = weno_face(f[pidx(i, j - 2, pit)], f[pidx(i, j - 1, pit)], f[id], f[pidx(i, j + 1, pit)], gt0(am));
    }
    // The p faces in two halves, so that the E_x-independent one runs beside the Poisson
    // solve: part 4 forms both upwind candidates (fp and, as scratch, Rp, which the
    // limiter rewrites later in the stage); part 8, once E_x is known, the velocity and the
    // choice.
    if ((part & 4) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np) {
        double vr, vl;
        weno_face_both(f[pidx(i, j - 2, pit)], f[pidx(i, j - 1, pit)], f[id], f[pidx(i, j + 1, pit)], vr, vl);
        P.fp[id] = vr;
        P.Rp[id] = vl;
    }
    if ((part & 8) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np) {
        const RunFields &F = fields[P.run];
        double Em = P.q * patch_efield(P, F, i);
        double am = Em - P.cc * P.dx_inv * (g[pidx(i + 1, j, pit)] - g[id]);
        P.ep[id] = am;
        if (!gt0(am)) P.fp[id] = P.Rp[id];
    }
}

// High-order fluxes for stage `step` and, on stage 0, the donor-cell low-order fluxes
// (Rectangle.cpp:1313-1394).  Coarse faces on a coarse/fine interface are skipped here
// and written by the interface kernel.
__global__ void k64_flux(const P64 *patches, const TileRef *tiles, int step, int use_f0, int part) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    const double *f = use_f0 ? P.f0 : P.f1;
    const double w3 = 1 / 48.0;
    if ((part & 1) && i >= 0 && i <= P.nx && j >= -1 && j <= P.np && !(P.ifx && P.ifx[id])) {
        double am = P.ex[id], ap1 = P.ex[id + 1], am1 = P.ex[id - 1];
        double fm = P.fx[id], fp1 = P.fx[id + 1], fm1 = P.fx[id - 1];
        P.FxH[step][id] = P.dx_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
        if (step == 0) P.FxL[id] = P.dx_inv * ((gt0(am) ? f[id - pit] : f[id]) * am);
    }
    if ((part & 2) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np && !(P.ifp && P.ifp[id])) {
        double am = P.ep[id], ap1 = P.ep[id + pit], am1 = P.ep[id - pit];
        double fm = P.fp[id], fp1 = P.fp[id + pit], fm1 = P.fp[id - pit];
        P.FpH[step][id] = P.dp_inv * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
        if (step == 0) P.FpL[id] = P.dp_inv * ((gt0(am) ? f[id - 1] : f[id]) * am);
    }
}

__device__ __forceinline__ bool active_face(const P64 &P, int i, int j) {
    return i >= P.xm && i < P.xp && j >= P.pm && j < P.pp;
}

// Stage flux combination (Rectangle.cpp:1396-1517) over the whole padded block, and the
// low-order solution f2 = f0 + div(LS) on the interior in the reference's accumulation
// order (Rectangle.cpp:1518-1534).  RK coefficients arrive pre-multiplied by dt.
__global__ void k64_ds_f2(const P64 *patches, const TileRef *tiles, const double *params, int s) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < -2 || j < -2) return;
    const double *a = params + param_base(P.run, s);
    const double asum = a[6];
    double hx, hp;
    hx = a[0] * P.FxH[0][id];
    hp = a[0] * P.FpH[0][id];
    for (int k = 1; k <= s; k++) {
        if (s == 5 && k == 1) continue;  // b_1 = 0 (Rectangle.cpp:1494)
        hx = hx + a[k] * P.FxH[k][id];
        hp = hp + a[k] * P.FpH[k][id];
    }
    double lsx = asum * P.FxL[id];
    double lsp = asum * P.FpL[id];
    P.FxDS[id] = hx - lsx;
    P.FpDS[id] = hp - lsp;
    if (i >= 0 && i < P.nx && j >= 0 && j < P.np) {
        double v = P.f0[id];
        if (active_face(P, i, j)) v += lsx;
        if (active_face(P, i, j)) v += lsp;
        if (active_face(P, i, j + 1)) v -= asum * P.FpL[id + 1];
        if (active_face(P, i + 1, j)) v -= asum * P.FxL[id + pit];
        P.f2[id] = v;
    }
}

// Zalesak R+/R- on i in [-1,nx], j in [-1,np] (Rectangle.cpp:1536-1579).
__global__ void k64_limR(const P64 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < -1 || i > P.nx || j < -1 || j > P.np) return;
    const double *DX = P.FxDS, *DP = P.FpDS, *f0 = P.f0, *f2 = P.f2;
    double dxi = DX[id], dxn = DX[id + pit], dpi = DP[id], dpn = DP[id + 1];
    double Pp = vmax0(dxi) - vmin0(dxn) + vmax0(dpi) - vmin0(dpn);
    double Pm = vmax0(dxn) - vmin0(dxi) + vmax0(dpn) - vmin0(dpi);
    double c0 = f0[id], c2 = f2[id];
    double w1ma = vmax(c0, c2);
    double w2ma = vmax(f0[id + pit], f2[id + pit]);
    double w3ma = vmax(f0[id - pit], f2[id - pit]);
    double w4ma = vmax(f0[id + 1], f2[id + 1]);
    double w5ma = vmax(f0[id - 1], f2[id - 1]);
    double wMax = vmax(w1ma, vmax(w2ma, vmax(w3ma, vmax(w4ma, w5ma))));
    double w1mi = vmin(c0, c2);
    double w2mi = vmin(f0[id + pit], f2[id + pit]);
    double w3mi = vmin(f0[id - pit], f2[id - pit]);
    double w4mi = vmin(f0[id + 1], f2[id + 1]);
    double w5mi = vmin(f0[id - 1], f2[id - 1]);
    double wMin = vmin(w1mi, vmin(w2mi, vmin(w3mi, vmin(w4mi, w5mi))));
    double Qm = -wMin + c2;
    double Qp = wMax - c2;
    // min(1, Q/P) is 1 whenever Q >= P and P is finite: the quotient (Q infinite
    // included) is then >= 1 however it rounds.  Every other case, NaN and infinite P
    // among them, takes the division as written.  Most cells of a smooth solution take
    // the first branch and skip the division (about ten FP64 instructions).
    constexpr double kMaxFinite = 1.7976931348623157e308;
    P.Rp[id] = gt0(Pp) ? ((Qp >= Pp && Pp <= kMaxFinite) ? 1.0 : vmin(1.0, Qp / Pp)) : 0.0;
    P.Rm[id] = gt0(Pm) ? ((Qm >= Pm && Pm <= kMaxFinite) ? 1.0 : vmin(1.0, Qm / Pm)) : 0.0;
}

// Limiter coefficients on interior faces, 1 elsewhere (Rectangle.cpp:1581-1594).
__global__ void k64_limC(const P64 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < -2 || j < -2) return;
    double cx = 1.0, cp = 1.0;
    if (i >= 1 && i < P.nx && j >= 0 && j < P.np) {
        const double *Rp = P.Rp, *Rm = P.Rm;
        cx = gt0(P.FxDS[id]) ? vmin(Rp[id], Rm[id - pit]) : vmin(Rp[id - pit], Rm[id]);
        cp = gt0(P.FpDS[id]) ? vmin(Rp[id], Rm[id - 1]) : vmin(Rp[id - 1], Rm[id]);
    }
    P.Cx[id] = cx;
    P.Cp[id] = cp;
}

// Antidiffusive update f1 = f2 + div(C * DS) (Rectangle.cpp:1595-1612).
__global__ void k64_update(const P64 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < 0 || i >= P.nx || j < 0 || j >= P.np) return;
    double v = P.f2[id];
    if (active_face(P, i, j)) v += P.Cx[id] * P.FxDS[id];
    if (active_face(P, i, j)) v += P.Cp[id] * P.FpDS[id];
    if (active_face(P, i, j + 1)) v -= P.Cp[id + 1] * P.FpDS[id + 1];
    if (active_face(P, i + 1, j)) v -= P.Cx[id + pit] * P.FxDS[id + pit];
    P.f1[id] = v;
}

// Last stage: f0 = f1 over the padded block (Rectangle.cpp:1614-1621).
__global__ void k64_copy10(const P64 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE_PROLOGUE
    if (i < -2 || j < -2) return;
    P.f0[id] = P.f1[id];
}

}  // namespace VX_FCT64_NS

// --------------------------------------------------------------------------------
void VX_FCT64_LAUNCH(const FctLaunch &L, int sub) {
    using namespace VX_FCT64_NS;
    dim3 blk(L.tile_j ? L.tile_j : 32, L.tile_i ? L.tile_i : 8);
    const P64 *pp = (const P64 *)L.patches;
    if (L.ntiles == 0) return;
    switch (sub) {
        case kSubGamma:
            vx_launch(k64_gamma, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.fields);
            break;
        case kSubFaces:
            vx_launch(k64_faces, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.fields, L.use_f0, L.part ? L.part : 3);
            break;
        case kSubFlux:
            vx_launch(k64_flux, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.step, L.use_f0, L.part ? L.part : 3);
            break;
        case kSubDsF2:
            vx_launch(k64_ds_f2, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.params, L.step);
            break;
        case kSubLimR:
            vx_launch(k64_limR, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubLimC:
            vx_launch(k64_limC, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubUpdate:
            vx_launch(k64_update, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubCopy10:
            vx_launch(k64_copy10, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
    }
}

}  // namespace vx
