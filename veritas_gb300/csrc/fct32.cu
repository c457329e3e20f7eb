// FP32 precision form of the per-patch FCT Runge-Kutta sub-steps
// (Rectangle::FCTTimeStep, Rectangle.cpp:1255-1623).
//
// Same sub-step decomposition, tile walk and face windows as the FP64 kernels; the
// arithmetic differs where FP32 needs it:
//   * f is stored scaled by the run's fnorm (1 / the peak of the initial distribution),
//     so every plane stays far inside FP32 range; the FCT update is linear in f and its
//     limiter is scale free, so nothing else changes;
//   * momenta are carried as p / (m c) and A^2 as q^2 A^2 / (m c)^2, so the Lorentz
//     factor is sqrt(1 + p^2 + a^2) in dimensionless FP32;
//   * the velocity differences of the reference, c^2 m (gamma(p_{j+1}) - gamma(p_j)) / dp
//     and c^2 m (gamma(A_{i+1}) - gamma(A_i)) / dx, are evaluated in the rationalised
//     form (p_{j+1}^2 - p_j^2) / (gamma_{j+1} + gamma_j), which has no cancellation, so
//     the face velocities keep FP32 relative accuracy (the direct difference of two
//     Lorentz factors near 1 would lose four digits).
// Compiled with fused multiply-add allowed.
#include <cuda_runtime.h>
#include "vx_kernels.hpp"

namespace vx {

using P32 = PatchT<float>;

// Quotients and square roots of the FP32 kernels use the hardware approximations
// (__fdividef: within 2 ulp for divisors below 2^126, which every divisor here is; and
// s * rsqrtf(s) for s >= 1); the precision form's stated error includes them.
__device__ __forceinline__ float sqrt_ge1(float s) { return s * rsqrtf(s); }

// WENO-type face value (Rectangle.cpp:980-1030) with the regulariser `mm`: the
// reference's 1e-10 carried into the scaled units of the smoothness indicators, floored
// at 1e-30 so that it stays a normal FP32 number (it only matters where f vanishes).
__device__ __forceinline__ float weno32(float f1, float f2, float f3, float f4, bool right, float mm) {
    const float c6 = 1.0f / 6.0f;
    const float c43 = 4.0f / 3.0f;
    float fL = c6 * (-f1 + 5.0f * f2 + 2.0f * f3);
    float fR = c6 * (2.0f * f2 + 5.0f * f3 - f4);
    float AL = f1 - 2.0f * f2 + f3;
    float BL = f3 - f1;
    float AR = f2 - 2.0f * f3 + f4;
    float BR = f4 - f2;
    float bL = c43 * (AL * AL) + 0.5f * AL * BL + 0.25f * (BL * BL);
    float bR = c43 * (AR * AR) - 0.5f * AR * BR + 0.25f * (BR * BR);
    // oL / (oL + oR) with o = 0.5 / (mm + b)^2, as a ratio that cannot underflow
    float rr = __fdividef(mm + bL, mm + bR);
    float wL = __fdividef(1.0f, 1.0f + rr * rr);  // rr^2 = inf gives wL = 0, its limit
    float wR = 1.0f - wL;
    float wL0 = wL * (0.75f + wL * (wL - 0.5f));
    float wR0 = wR * (0.75f + wR * (wR - 0.5f));
    float pick = right ? fmaxf(wL0, wR0) : fminf(wL0, wR0);
    float fwl = __fdividef(pick, wL0 + wR0);  // wL0 + wR0 >= 0.75
    return fwl * fL + (1.0f - fwl) * fR;
}

// Dimensionless momentum of p-face j, q^2 A^2 / (m c)^2 at the finest face under x-face
// i, and q times the rtb-average of E_x under coarse cell i (Rectangle::GetEfield,
// Rectangle.cpp:1055-1067), all from FP32 copies.
__device__ __forceinline__ float mom32(const P32 &P, int j) { return fmaf(P.dpnf, (float)(j + P.p_pos), P.pminf); }
__device__ __forceinline__ float asq32(const P32 &P, const RunFields &F, int i) {
    int x = P.rtb * (i + P.x_pos);
    x = x < 0 ? 0 : (x > F.n ? F.n : x);
    return P.a2nf * F.asq32[x];
}
__device__ __forceinline__ float qefield32(const P32 &P, const RunFields &F, int i) {
    int x = P.rtb * (i + P.x_pos);
    float t = 0.0f;
    for (int k = 0; k < P.rtb; k++) {
        int y = x + k;
        y = (y > -1) ? y : (y + F.n);
        y = (y < F.n) ? y : (y - F.n);
        t += F.efin32[y];
    }
    return P.qf * (t * (1.0f / (float)P.rtb));  // rtb is a power of two
}

#define VX_TILE32                                         \
    const TileRef t = tiles[blockIdx.x];                  \
    const P32 &P = patches[t.patch];                      \
    const int i = t.i0 + (int)threadIdx.y;                \
    const int j = t.j0 + (int)threadIdx.x;                \
    if (i > P.nx + 1 || j > P.np + 1) return;             \
    const int pit = P.pitch;                              \
    const int id = pidx(i, j, pit);

// Lorentz factor at (x-face i, p-face j), i in [-1,nx+1], j in [-1,np+1].
__global__ void k32_gamma(const P32 *patches, const TileRef *tiles, const RunFields *fields) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < -1 || j < -1) return;
    const RunFields &F = fields[P.run];
    const float a = asq32(P, F, i);
    const float p = mom32(P, j);
    P.gam[id] = sqrtf(1.0f + p * p + a);
}

__global__ void k32_faces(const P32 *patches, const TileRef *tiles, const RunFields *fields, int use_f0, int part) {
    VX_PDL_WAIT();
    VX_TILE32
    const float *f = use_f0 ? P.f0 : P.f1;
    const float *g = P.gam;
    const float mm = P.weno_eps;
    if ((part & 1) && i >= 0 && i <= P.nx && j >= -1 && j <= P.np) {
        const float p0 = mom32(P, j), p1 = mom32(P, j + 1);
        const float dg = P.dpnf * (p1 + p0) / (g[pidx(i, j + 1, pit)] + g[id]);
        const float am = P.kxf * dg;
        P.ex[id] = am;
        P.fx[id] = weno32(f[pidx(i - 2, j, pit)], f[pidx(i - 1, j, pit)], f[id], f[pidx(i + 1, j, pit)], am > 0.0f, mm);
    }
    if ((part & 2) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np) {
        const RunFields &F = fields[P.run];
        const float Em = qefield32(P, F, i);
        const float a0 = asq32(P, F, i), a1 = asq32(P, F, i + 1);
        const float dg = (a1 - a0) / (g[pidx(i + 1, j, pit)] + g[id]);
        const float am = Em - P.kpf * dg;
        P.ep[id] = am;
        P.fp[id] = weno32(f[pidx(i, j - 2, pit)], f[pidx(i, j - 1, pit)], f[id], f[pidx(i, j + 1, pit)], am > 0.0f, mm);
    }
}

__global__ void k32_flux(const P32 *patches, const TileRef *tiles, int step, int use_f0, int part) {
    VX_PDL_WAIT();
    VX_TILE32
    const float *f = use_f0 ? P.f0 : P.f1;
    const float w3 = 1.0f / 48.0f;
    const float dxi = P.dxif, dpi = P.dpif;
    if ((part & 1) && i >= 0 && i <= P.nx && j >= -1 && j <= P.np && !(P.ifx && P.ifx[id])) {
        float am = P.ex[id], ap1 = P.ex[id + 1], am1 = P.ex[id - 1];
        float fm = P.fx[id], fp1 = P.fx[id + 1], fm1 = P.fx[id - 1];
        P.FxH[step][id] = dxi * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
        if (step == 0) P.FxL[id] = dxi * ((am > 0.0f ? f[id - pit] : f[id]) * am);
    }
    if ((part & 2) && i >= -1 && i <= P.nx && j >= 0 && j <= P.np && !(P.ifp && P.ifp[id])) {
        float am = P.ep[id], ap1 = P.ep[id + pit], am1 = P.ep[id - pit];
        float fm = P.fp[id], fp1 = P.fp[id + pit], fm1 = P.fp[id - pit];
        P.FpH[step][id] = dpi * (fm * am + w3 * (fp1 - fm1) * (ap1 - am1));
        if (step == 0) P.FpL[id] = dpi * ((am > 0.0f ? f[id - 1] : f[id]) * am);
    }
}

__device__ __forceinline__ bool active32(const P32 &P, int i, int j) {
    return i >= P.xm && i < P.xp && j >= P.pm && j < P.pp;
}

__global__ void k32_ds_f2(const P32 *patches, const TileRef *tiles, const float *params, int s) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < -2 || j < -2) return;
    const float *a = params + param_base(P.run, s);
    const float asum = a[6];
    float hx = a[0] * P.FxH[0][id];
    float hp = a[0] * P.FpH[0][id];
    for (int k = 1; k <= s; k++) {
        if (s == 5 && k == 1) continue;  // b_1 = 0 (Rectangle.cpp:1494)
        hx += a[k] * P.FxH[k][id];
        hp += a[k] * P.FpH[k][id];
    }
    const float lsx = asum * P.FxL[id];
    const float lsp = asum * P.FpL[id];
    P.FxDS[id] = hx - lsx;
    P.FpDS[id] = hp - lsp;
    if (i >= 0 && i < P.nx && j >= 0 && j < P.np) {
        float v = P.f0[id];
        if (active32(P, i, j)) v += lsx;
        if (active32(P, i, j)) v += lsp;
        if (active32(P, i, j + 1)) v -= asum * P.FpL[id + 1];
        if (active32(P, i + 1, j)) v -= asum * P.FxL[id + pit];
        P.f2[id] = v;
    }
}

__global__ void k32_limR(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < -1 || i > P.nx || j < -1 || j > P.np) return;
    const float *DX = P.FxDS, *DP = P.FpDS, *f0 = P.f0, *f2 = P.f2;
    float dxi = DX[id], dxn = DX[id + pit], dpi = DP[id], dpn = DP[id + 1];
    float Pp = fmaxf(0.0f, dxi) - fminf(0.0f, dxn) + fmaxf(0.0f, dpi) - fminf(0.0f, dpn);
    float Pm = fmaxf(0.0f, dxn) - fminf(0.0f, dxi) + fmaxf(0.0f, dpn) - fminf(0.0f, dpi);
    float c0 = f0[id], c2 = f2[id];
    float wMax = fmaxf(fmaxf(c0, c2), fmaxf(fmaxf(f0[id + pit], f2[id + pit]),
                 fmaxf(fmaxf(f0[id - pit], f2[id - pit]), fmaxf(fmaxf(f0[id + 1], f2[id + 1]), fmaxf(f0[id - 1], f2[id - 1])))));
    float wMin = fminf(fminf(c0, c2), fminf(fminf(f0[id + pit], f2[id + pit]),
                 fminf(fminf(f0[id - pit], f2[id - pit]), fminf(fminf(f0[id + 1], f2[id + 1]), fminf(f0[id - 1], f2[id - 1])))));
    float Qm = -wMin + c2;
    float Qp = wMax - c2;
    P.Rp[id] = Pp > 0.0f ? fminf(1.0f, Qp / Pp) : 0.0f;
    P.Rm[id] = Pm > 0.0f ? fminf(1.0f, Qm / Pm) : 0.0f;
}

__global__ void k32_limC(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < -2 || j < -2) return;
    float cx = 1.0f, cp = 1.0f;
    if (i >= 1 && i < P.nx && j >= 0 && j < P.np) {
        const float *Rp = P.Rp, *Rm = P.Rm;
        cx = P.FxDS[id] > 0.0f ? fminf(Rp[id], Rm[id - pit]) : fminf(Rp[id - pit], Rm[id]);
        cp = P.FpDS[id] > 0.0f ? fminf(Rp[id], Rm[id - 1]) : fminf(Rp[id - 1], Rm[id]);
    }
    P.Cx[id] = cx;
    P.Cp[id] = cp;
}

__global__ void k32_update(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < 0 || i >= P.nx || j < 0 || j >= P.np) return;
    float v = P.f2[id];
    if (active32(P, i, j)) v += P.Cx[id] * P.FxDS[id];
    if (active32(P, i, j)) v += P.Cp[id] * P.FpDS[id];
    if (active32(P, i, j + 1)) v -= P.Cp[id + 1] * P.FpDS[id + 1];
    if (active32(P, i + 1, j)) v -= P.Cx[id + pit] * P.FxDS[id + pit];
    P.f1[id] = v;
}

__global__ void k32_copy10(const P32 *patches, const TileRef *tiles) {
    VX_PDL_WAIT();
    VX_TILE32
    if (i < -2 || j < -2) return;
    P.f0[id] = P.f1[id];
}


// ---------------------------------------------------------------- fused face + flux
// One warp per strip tile: Lorentz factors, face velocities and WENO values are formed in
// registers and consumed there (neighbours through shuffles), so neither gamma nor the
// face planes go to HBM.  The fluxes are those of k32_faces / k32_flux; face values
// outside the ranges the separate kernels write (x: i in [0, nx], j in [-1, np];
// p: i in [-1, nx], j in [0, np]) are zero, as the planes they read are.

// x direction: a warp covers kXCols output columns j0 .. j0+29 (its 32 lanes hold the
// face values of j0-1 .. j0+30) over kStripRows rows; rows are independent in x.
__global__ void k32_xflux(const P32 *patches, const TileRef *tiles, int ntiles, const RunFields *fields, int step,
                          int use_f0) {
    VX_PDL_WAIT();
    const int wt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wt >= ntiles) return;
    const int lane = threadIdx.x & 31;
    const TileRef t = tiles[wt];
    const P32 &P = patches[t.patch];
    const int pit = P.pitch;
    const float *f = use_f0 ? P.f0 : P.f1;
    const RunFields &F = fields[P.run];
    const int jj = t.j0 - 1 + lane;
    const bool col_ok = jj >= -1 && jj <= P.np;
    const float p0 = mom32(P, jj), p1 = mom32(P, jj + 1);
    const float w3 = 1.0f / 48.0f;
    const unsigned full = 0xffffffffu;
    for (int r = 0; r < kStripRows; r++) {
        const int i = t.i0 + r;
        if (i > P.nx) break;  // warp-uniform
        float am = 0.0f, fv = 0.0f;
        if (col_ok) {
            const float a = asq32(P, F, i);
            const float g0 = sqrt_ge1(1.0f + p0 * p0 + a), g1 = sqrt_ge1(1.0f + p1 * p1 + a);
            am = P.kxf * __fdividef(P.dpnf * (p1 + p0), g1 + g0);
            const int id = pidx(i, jj, pit);
            fv = weno32(f[id - 2 * pit], f[id - pit], f[id], f[id + pit], am > 0.0f, P.weno_eps);
        }
        const float am1 = __shfl_up_sync(full, am, 1), ap1 = __shfl_down_sync(full, am, 1);
        const float fm1 = __shfl_up_sync(full, fv, 1), fp1 = __shfl_down_sync(full, fv, 1);
        if (lane < 1 || lane > kXCols || !col_ok) continue;
        const int id = pidx(i, jj, pit);
        if (P.ifx && P.ifx[id]) continue;
        P.FxH[step][id] = P.dxif * (fv * am + w3 * (fp1 - fm1) * (ap1 - am1));
        if (step == 0) P.FxL[id] = P.dxif * ((am > 0.0f ? f[id - pit] : f[id]) * am);
    }
}

// p direction: a warp covers 32 columns over kStripRows output rows, walking down with
// the face values of the previous and next rows in registers.
__device__ __forceinline__ void pface32(const P32 &P, const RunFields &F, const float *f, int i, int j, float p,
                                        bool col_ok, float &am, float &fv) {
    am = 0.0f;
    fv = 0.0f;
    if (!col_ok || i < -1 || i > P.nx) return;
    const float a0 = asq32(P, F, i), a1 = asq32(P, F, i + 1);
    const float g0 = sqrt_ge1(1.0f + p * p + a0), g1 = sqrt_ge1(1.0f + p * p + a1);
    am = qefield32(P, F, i) - P.kpf * __fdividef(a1 - a0, g1 + g0);
    const int id = pidx(i, j, P.pitch);
    fv = weno32(f[id - 2], f[id - 1], f[id], f[id + 1], am > 0.0f, P.weno_eps);
}

__global__ void k32_pflux(const P32 *patches, const TileRef *tiles, int ntiles, const RunFields *fields, int step,
                          int use_f0) {
    VX_PDL_WAIT();
    const int wt = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wt >= ntiles) return;
    const int lane = threadIdx.x & 31;
    const TileRef t = tiles[wt];
    const P32 &P = patches[t.patch];
    const float *f = use_f0 ? P.f0 : P.f1;
    const RunFields &F = fields[P.run];
    const int j = t.j0 + lane;
    const bool col_ok = j >= 0 && j <= P.np;
    const float p = mom32(P, j);
    const float w3 = 1.0f / 48.0f;
    float amA, fvA, amB, fvB;  // rows i-1 and i
    pface32(P, F, f, t.i0 - 1, j, p, col_ok, amA, fvA);
    pface32(P, F, f, t.i0, j, p, col_ok, amB, fvB);
    for (int r = 0; r < kStripRows; r++) {
        const int i = t.i0 + r;
        if (i > P.nx) break;
        float amC, fvC;  // row i+1
        pface32(P, F, f, i + 1, j, p, col_ok, amC, fvC);
        if (col_ok && !(P.ifp && P.ifp[pidx(i, j, P.pitch)])) {
            const int id = pidx(i, j, P.pitch);
            P.FpH[step][id] = P.dpif * (fvB * amB + w3 * (fvC - fvA) * (amC - amA));
            if (step == 0) P.FpL[id] = P.dpif * ((amB > 0.0f ? f[id - 1] : f[id]) * amB);
        }
        amA = amB;
        fvA = fvB;
        amB = amC;
        fvB = fvC;
    }
}

void launch_fct32_substep(const FctLaunch &L, int sub) {
    dim3 blk(L.tile_j ? L.tile_j : 32, L.tile_i ? L.tile_i : 8);
    const P32 *pp = (const P32 *)L.patches;
    if (L.ntiles == 0) return;
    switch (sub) {
        case kSubGamma:
            vx_launch(k32_gamma, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.fields);
            break;
        case kSubFaces:
            vx_launch(k32_faces, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.fields, L.use_f0, L.part ? L.part : 3);
            break;
        case kSubFlux:
            vx_launch(k32_flux, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.step, L.use_f0, L.part ? L.part : 3);
            break;
        case kSubDsF2:
            vx_launch(k32_ds_f2, L.ntiles, blk, 0, L.stream, pp, L.tiles, L.params32, L.step);
            break;
        case kSubLimR:
            vx_launch(k32_limR, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubLimC:
            vx_launch(k32_limC, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubUpdate:
            vx_launch(k32_update, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubCopy10:
            vx_launch(k32_copy10, L.ntiles, blk, 0, L.stream, pp, L.tiles);
            break;
        case kSubXFlux:
            if (L.nxtiles) vx_launch(k32_xflux, (L.nxtiles + 3) / 4, 128, 0, L.stream, pp, L.xtiles, L.nxtiles, L.fields, L.step, L.use_f0);
            break;
        case kSubPFlux:
            if (L.nptiles) vx_launch(k32_pflux, (L.nptiles + 3) / 4, 128, 0, L.stream, pp, L.ptiles, L.nptiles, L.fields, L.step, L.use_f0);
            break;
    }
}

}  // namespace vx
