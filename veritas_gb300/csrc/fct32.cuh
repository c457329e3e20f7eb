// FP32 precision form of the per-patch FCT Runge-Kutta sub-steps
// (Rectangle::FCTTimeStep, Rectangle.cpp:1255-1623): the device bodies, one tile or strip
// per call, shared by the per-sub-step kernels (fct32.cu) and the persistent stage kernel
// (stage32.cu).  Both translation units are compiled with fused multiply-add allowed, and
// the bodies are the same source, so the two launch forms give the same bits.
//
// Same sub-steps and face windows as the FP64 kernels (gamma, faces and fluxes fused per
// direction; the cell-wise sub-steps with 128-bit accesses); the arithmetic differs where
// FP32 needs it:
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
#pragma once
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

__device__ __forceinline__ bool active32(const P32 &P, int i, int j) {
    return i >= P.xm && i < P.xp && j >= P.pm && j < P.pp;
}

// ---------------------------------------------------------------- streaming sub-steps
// The cell-wise sub-steps move whole planes with 128-bit accesses: a thread owns four
// consecutive p cells (j .. j+3) of one row, a tile is tile_i rows by 128 p cells.  Tiles
// start at j0 = -2 + 128 k, so j + 2 is a multiple of 4 and, with the pitch a multiple of
// 8 and every plane 16-byte aligned, each thread's four cells are one aligned float4.  The
// p neighbours past the four (j - 1, j + 4) are scalar loads, made only when a valid cell
// needs them (they are then inside the row).  Each body handles the thread (tx, row) of
// tile t: lane tx of the tile's 32 columns of four cells, row `row` of its tile_i rows.
#define VX_VTILE32                                        \
    const P32 &P = patches[t.patch];                      \
    const int i = t.i0 + row;                             \
    const int j = t.j0 + 4 * tx;                          \
    if (i > P.nx + 1 || j > P.np + 1) return;             \
    const int pit = P.pitch;                              \
    const int id = pidx(i, j, pit);

struct V4 {
    float v[4];
};
__device__ __forceinline__ V4 ld4(const float *p) {
    const float4 q = *reinterpret_cast<const float4 *>(p);
    return {{q.x, q.y, q.z, q.w}};
}
// Stores the elements e with lo <= j + e < hi (one 128-bit store when all four are).
__device__ __forceinline__ void st4(float *p, const V4 &x, int j, int lo, int hi) {
    if (j >= lo && j + 3 < hi) {
        *reinterpret_cast<float4 *>(p) = make_float4(x.v[0], x.v[1], x.v[2], x.v[3]);
        return;
    }
#pragma unroll
    for (int e = 0; e < 4; e++)
        if (j + e >= lo && j + e < hi) p[e] = x.v[e];
}

// RK flux combination and low-order solution (Rectangle.cpp:1396-1534): DS over the
// padded block, f2 over the interior.
__device__ __forceinline__ void ds_f2_32(const P32 *patches, const TileRef t, int tx, int row, const float *params,
                                         int s) {
    VX_VTILE32
    const float *a = params + param_base(P.run, s);
    const float asum = a[6];
    V4 hx = ld4(P.FxH[0] + id), hp = ld4(P.FpH[0] + id);
#pragma unroll
    for (int e = 0; e < 4; e++) {
        hx.v[e] = a[0] * hx.v[e];
        hp.v[e] = a[0] * hp.v[e];
    }
    for (int k = 1; k <= s; k++) {
        if (s == 5 && k == 1) continue;  // b_1 = 0 (Rectangle.cpp:1494)
        const V4 gx = ld4(P.FxH[k] + id), gp = ld4(P.FpH[k] + id);
        const float ak = a[k];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            hx.v[e] += ak * gx.v[e];
            hp.v[e] += ak * gp.v[e];
        }
    }
    const V4 lx = ld4(P.FxL + id), lp = ld4(P.FpL + id);
    V4 dx, dp, lsx, lsp;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        lsx.v[e] = asum * lx.v[e];
        lsp.v[e] = asum * lp.v[e];
        dx.v[e] = hx.v[e] - lsx.v[e];
        dp.v[e] = hp.v[e] - lsp.v[e];
    }
    st4(P.FxDS + id, dx, j, -2, P.np + 2);
    st4(P.FpDS + id, dp, j, -2, P.np + 2);
    if (i < 0 || i >= P.nx || j + 3 < 0 || j >= P.np) return;
    const V4 f0 = ld4(P.f0 + id), lxn = ld4(P.FxL + id + pit);
    const float lp4 = (j + 3 < P.np) ? P.FpL[id + 4] : 0.0f;  // j + 4 <= np
    V4 f2;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int je = j + e;
        float v = f0.v[e];
        if (active32(P, i, je)) v += lsx.v[e];
        if (active32(P, i, je)) v += lsp.v[e];
        if (active32(P, i, je + 1)) v -= asum * (e < 3 ? lp.v[e + 1] : lp4);
        if (active32(P, i + 1, je)) v -= asum * lxn.v[e];
        f2.v[e] = v;
    }
    st4(P.f2 + id, f2, j, 0, P.np);
}

// min(1, Q / P) for P > 0, else 0 (Q >= 0: a stencil extremum minus the centre value).
// Q >= P gives 1 without a quotient; otherwise the hardware reciprocal (within 2 ulp),
// except for a subnormal P, where it is not defined and IEEE division is used.
__device__ __forceinline__ float limiter_ratio(float Q, float P) {
    if (!(P > 0.0f)) return 0.0f;
    if (Q >= P) return 1.0f;
    return fminf(1.0f, P >= 1.17549435e-38f ? __fdividef(Q, P) : Q / P);
}

// Zalesak R+ and R- (Rectangle.cpp:1536-1582), cells i in [-1, nx], j in [-1, np].
__device__ __forceinline__ void limR32(const P32 *patches, const TileRef t, int tx, int row) {
    VX_VTILE32
    if (i < -1 || i > P.nx || j + 3 < -1 || j > P.np) return;
    const float *DX = P.FxDS, *DP = P.FpDS, *f0 = P.f0, *f2 = P.f2;
    const V4 dxi = ld4(DX + id), dxn = ld4(DX + id + pit), dpi = ld4(DP + id);
    const V4 a0 = ld4(f0 + id), a2 = ld4(f2 + id);
    const V4 u0 = ld4(f0 + id + pit), u2 = ld4(f2 + id + pit);
    const V4 d0 = ld4(f0 + id - pit), d2 = ld4(f2 + id - pit);
    const bool lo_ok = j >= -1, hi_ok = j + 3 <= P.np;  // element 0 / element 3 valid
    const float l0 = lo_ok ? f0[id - 1] : 0.0f, l2 = lo_ok ? f2[id - 1] : 0.0f;
    const float r0 = hi_ok ? f0[id + 4] : 0.0f, r2 = hi_ok ? f2[id + 4] : 0.0f;
    const float dp4 = hi_ok ? DP[id + 4] : 0.0f;
    V4 rp, rm;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const float dpn = e < 3 ? dpi.v[e + 1] : dp4;
        const float Pp = fmaxf(0.0f, dxi.v[e]) - fminf(0.0f, dxn.v[e]) + fmaxf(0.0f, dpi.v[e]) - fminf(0.0f, dpn);
        const float Pm = fmaxf(0.0f, dxn.v[e]) - fminf(0.0f, dxi.v[e]) + fmaxf(0.0f, dpn) - fminf(0.0f, dpi.v[e]);
        const float c0 = a0.v[e], c2 = a2.v[e];
        const float lf0 = e > 0 ? a0.v[e - 1] : l0, lf2 = e > 0 ? a2.v[e - 1] : l2;
        const float rf0 = e < 3 ? a0.v[e + 1] : r0, rf2 = e < 3 ? a2.v[e + 1] : r2;
        const float wMax = fmaxf(fmaxf(c0, c2), fmaxf(fmaxf(u0.v[e], u2.v[e]),
                           fmaxf(fmaxf(d0.v[e], d2.v[e]), fmaxf(fmaxf(rf0, rf2), fmaxf(lf0, lf2)))));
        const float wMin = fminf(fminf(c0, c2), fminf(fminf(u0.v[e], u2.v[e]),
                           fminf(fminf(d0.v[e], d2.v[e]), fminf(fminf(rf0, rf2), fminf(lf0, lf2)))));
        const float Qm = -wMin + c2;
        const float Qp = wMax - c2;
        rp.v[e] = limiter_ratio(Qp, Pp);
        rm.v[e] = limiter_ratio(Qm, Pm);
    }
    st4(P.Rp + id, rp, j, -1, P.np + 1);
    st4(P.Rm + id, rm, j, -1, P.np + 1);
}

// Face coefficients C (Rectangle.cpp:1583-1594) over the padded block: 1 outside
// i in [1, nx), j in [0, np).
__device__ __forceinline__ void limC32(const P32 *patches, const TileRef t, int tx, int row) {
    VX_VTILE32
    V4 cx{{1.0f, 1.0f, 1.0f, 1.0f}}, cp{{1.0f, 1.0f, 1.0f, 1.0f}};
    if (i >= 1 && i < P.nx && j + 3 >= 0 && j < P.np) {
        const float *Rp = P.Rp, *Rm = P.Rm;
        const V4 rpi = ld4(Rp + id), rmi = ld4(Rm + id), rpd = ld4(Rp + id - pit), rmd = ld4(Rm + id - pit);
        const V4 dx = ld4(P.FxDS + id), dp = ld4(P.FpDS + id);
        const bool lo_ok = j >= 0;
        const float rpl = lo_ok ? Rp[id - 1] : 0.0f, rml = lo_ok ? Rm[id - 1] : 0.0f;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            if (j + e < 0 || j + e >= P.np) continue;
            const float rpm = e > 0 ? rpi.v[e - 1] : rpl, rmm = e > 0 ? rmi.v[e - 1] : rml;
            cx.v[e] = dx.v[e] > 0.0f ? fminf(rpi.v[e], rmd.v[e]) : fminf(rpd.v[e], rmi.v[e]);
            cp.v[e] = dp.v[e] > 0.0f ? fminf(rpi.v[e], rmm) : fminf(rpm, rmi.v[e]);
        }
    }
    st4(P.Cx + id, cx, j, -2, P.np + 2);
    st4(P.Cp + id, cp, j, -2, P.np + 2);
}

// Antidiffusive update (Rectangle.cpp:1595-1612), interior cells.
__device__ __forceinline__ void update32(const P32 *patches, const TileRef t, int tx, int row) {
    VX_VTILE32
    if (i < 0 || i >= P.nx || j + 3 < 0 || j >= P.np) return;
    const V4 f2 = ld4(P.f2 + id), cx = ld4(P.Cx + id), dx = ld4(P.FxDS + id), cp = ld4(P.Cp + id),
             dp = ld4(P.FpDS + id);
    const V4 cxn = ld4(P.Cx + id + pit), dxn = ld4(P.FxDS + id + pit);
    const bool hi_ok = j + 3 < P.np;  // element 3 valid: j + 4 <= np
    const float cp4 = hi_ok ? P.Cp[id + 4] : 0.0f, dp4 = hi_ok ? P.FpDS[id + 4] : 0.0f;
    V4 out;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int je = j + e;
        float v = f2.v[e];
        if (active32(P, i, je)) v += cx.v[e] * dx.v[e];
        if (active32(P, i, je)) v += cp.v[e] * dp.v[e];
        if (active32(P, i, je + 1)) v -= (e < 3 ? cp.v[e + 1] : cp4) * (e < 3 ? dp.v[e + 1] : dp4);
        if (active32(P, i + 1, je)) v -= cxn.v[e] * dxn.v[e];
        out.v[e] = v;
    }
    st4(P.f1 + id, out, j, 0, P.np);
}

// f0 = f1 over the padded block (Rectangle.cpp:1614-1621).
__device__ __forceinline__ void copy10_32(const P32 *patches, const TileRef t, int tx, int row) {
    VX_VTILE32
    st4(P.f0 + id, ld4(P.f1 + id), j, -2, P.np + 2);
}
#undef VX_VTILE32

// ---------------------------------------------------------------- fused face + flux
// One warp per strip tile: Lorentz factors, face velocities and WENO values are formed in
// registers and consumed there (neighbours through shuffles), so the FP32 form has no
// gamma or face planes at all.  The fluxes are the FP64 path's (k64_faces + k64_flux) in
// FP32; face values outside the reference's face ranges (x: i in [0, nx], j in [-1, np];
// p: i in [-1, nx], j in [0, np]) count as zero.  All 32 lanes of the warp call a strip
// body together (it shuffles across the warp).

// The descriptor and field-block values the p-direction body uses, read once into
// registers: its row loop stores to global memory, after which the compiler would
// otherwise reload every descriptor field it cannot prove unchanged (measured: the p
// kernel 32.5 -> 29.8 us on the 4096 x 512 case; the x kernel, with fewer fields in its
// loop, ran slower with the same change and keeps the descriptor reads).
struct FluxView {
    int nx, np, pit, rtb, x_pos, n;
    float dpnf, pminf, kpf, dpif, weno_eps, a2nf, qf, inv_rtb;
    const float *f, *asq, *efin;
    const uint8_t *ifp;
    float *FH, *FL;
    __device__ __forceinline__ FluxView(const P32 &P, const RunFields &F, int step, int use_f0) {
        nx = P.nx;
        np = P.np;
        pit = P.pitch;
        rtb = P.rtb;
        x_pos = P.x_pos;
        n = F.n;
        dpnf = P.dpnf;
        pminf = P.pminf;
        kpf = P.kpf;
        dpif = P.dpif;
        weno_eps = P.weno_eps;
        a2nf = P.a2nf;
        qf = P.qf;
        inv_rtb = 1.0f / (float)P.rtb;  // rtb is a power of two
        f = use_f0 ? P.f0 : P.f1;
        asq = F.asq32;
        efin = F.efin32;
        ifp = P.ifp;
        FH = P.FpH[step];
        FL = P.FpL;
    }
    // dimensionless momentum of p-face j (P.p_pos folded into the caller's j)
    __device__ __forceinline__ float mom(int jg) const { return fmaf(dpnf, (float)jg, pminf); }
    // q^2 A^2 / (m c)^2 at the finest face under x-face i
    __device__ __forceinline__ float asq_at(int i) const {
        int x = rtb * (i + x_pos);
        x = x < 0 ? 0 : (x > n ? n : x);
        return a2nf * asq[x];
    }
    // q times the rtb-average of E_x under coarse cell i (Rectangle::GetEfield,
    // Rectangle.cpp:1055-1067), periodic in x
    __device__ __forceinline__ float qe_at(int i) const {
        const int x = rtb * (i + x_pos);
        float t = 0.0f;
        for (int k = 0; k < rtb; k++) {
            int y = x + k;
            y = (y > -1) ? y : (y + n);
            y = (y < n) ? y : (y - n);
            t += efin[y];
        }
        return qf * (t * inv_rtb);
    }
};

// x direction: a warp covers kXCols output columns j0 .. j0+29 (its 32 lanes hold the
// face values of j0-1 .. j0+30) over kStripRows rows; rows are independent in x, and the
// four rows of f a face reads (i-2 .. i+1) slide down the strip, one new load per row.
__device__ __forceinline__ void xflux32(const P32 *patches, const TileRef t, int lane, const RunFields *fields,
                                       int step, int use_f0) {
    const P32 &P = patches[t.patch];
    const int pit = P.pitch;
    const float *f = use_f0 ? P.f0 : P.f1;
    const RunFields &F = fields[P.run];
    const int jj = t.j0 - 1 + lane;
    const bool col_ok = jj >= -1 && jj <= P.np;
    const float p0 = mom32(P, jj), p1 = mom32(P, jj + 1);
    const float w3 = 1.0f / 48.0f;
    const unsigned full = 0xffffffffu;
    // f at rows i-2, i-1, i of the first row (i0 >= 0, so all inside the padded block)
    float fa = 0.0f, fb = 0.0f, fc = 0.0f;
    if (col_ok) {
        const int id = pidx(t.i0, jj, pit);
        fa = f[id - 2 * pit];
        fb = f[id - pit];
        fc = f[id];
    }
    // q^2 A^2 / (m c)^2 of row i0 + k, formed once by lane k and taken by shuffle
    const float a_l = asq32(P, F, t.i0 + lane);
    for (int r = 0; r < kStripRows; r++) {
        const int i = t.i0 + r;
        if (i > P.nx) break;  // warp-uniform
        const int id = pidx(i, jj, pit);
        float am = 0.0f, fv = 0.0f, fd = 0.0f;
        const float a = __shfl_sync(full, a_l, r);
        if (col_ok) {
            fd = f[id + pit];  // row i+1 <= nx+1
            const float g0 = sqrt_ge1(1.0f + p0 * p0 + a), g1 = sqrt_ge1(1.0f + p1 * p1 + a);
            am = P.kxf * __fdividef(P.dpnf * (p1 + p0), g1 + g0);
            fv = weno32(fa, fb, fc, fd, am > 0.0f, P.weno_eps);
        }
        const float am1 = __shfl_up_sync(full, am, 1), ap1 = __shfl_down_sync(full, am, 1);
        const float fm1 = __shfl_up_sync(full, fv, 1), fp1 = __shfl_down_sync(full, fv, 1);
        if (lane >= 1 && lane <= kXCols && col_ok && !(P.ifx && P.ifx[id])) {
            P.FxH[step][id] = P.dxif * (fv * am + w3 * (fp1 - fm1) * (ap1 - am1));
            if (step == 0) P.FxL[id] = P.dxif * ((am > 0.0f ? fb : fc) * am);  // f[i-1] or f[i]
        }
        fa = fb;
        fb = fc;
        fc = fd;
    }
}

// p direction: a warp covers 32 columns over kStripRows output rows, walking down with
// the face values of the previous and next rows in registers.  Face row i reads a^2 and
// gamma at x-faces i and i+1; the i+1 pair is the next row's i pair, so it is carried.
struct PRow {
    float a, g;  // q^2 A^2 / (m c)^2 and gamma at the row's lower x-face
};
__device__ __forceinline__ void pface32(const FluxView &V, int i, int j, bool col_ok, const PRow &lo,
                                        const PRow &hi, float qe, float &am, float &fv) {
    am = 0.0f;
    fv = 0.0f;
    if (!col_ok || i < -1 || i > V.nx) return;
    am = qe - V.kpf * __fdividef(hi.a - lo.a, hi.g + lo.g);
    const int id = pidx(i, j, V.pit);
    const float *f = V.f;
    fv = weno32(f[id - 2], f[id - 1], f[id], f[id + 1], am > 0.0f, V.weno_eps);
}

// The row quantities — q^2 A^2 / (m c)^2 at x-faces i0-1 .. i0+rows+1 and q<E_x> of rows
// i0-1 .. i0+rows — are the same for every lane: lane k forms those of row i0-1+k once
// (k <= kStripRows + 2 < 32) and each row takes them by shuffle, instead of every lane
// forming every row's (their index clamping and the periodic E_x average were most of the
// kernel's integer instructions).
__device__ __forceinline__ void pflux32(const P32 *patches, const TileRef t, int lane, const RunFields *fields,
                                       int step, int use_f0) {
    const unsigned full = 0xffffffffu;
    const P32 &P = patches[t.patch];
    const FluxView V(P, fields[P.run], step, use_f0);
    const int j = t.j0 + lane;
    const bool col_ok = j >= 0 && j <= V.np;
    const float p = V.mom(j + P.p_pos);
    const float w3 = 1.0f / 48.0f;
    const int ir = t.i0 - 1 + lane;
    const float a_l = V.asq_at(ir);
    const float qe_l = (ir >= -1 && ir <= V.nx) ? V.qe_at(ir) : 0.0f;
    auto prow = [&](int i) {  // i - (i0 - 1) in 0 .. kStripRows + 2
        const float a = __shfl_sync(full, a_l, i - (t.i0 - 1));
        return PRow{a, sqrt_ge1(1.0f + p * p + a)};
    };
    auto qe = [&](int i) { return __shfl_sync(full, qe_l, i - (t.i0 - 1)); };
    PRow r0 = prow(t.i0 - 1), r1 = prow(t.i0), r2 = prow(t.i0 + 1);
    float amA, fvA, amB, fvB;  // rows i-1 and i
    pface32(V, t.i0 - 1, j, col_ok, r0, r1, qe(t.i0 - 1), amA, fvA);
    pface32(V, t.i0, j, col_ok, r1, r2, qe(t.i0), amB, fvB);
    const int rows = min(kStripRows, V.nx + 1 - t.i0);
    for (int r = 0; r < rows; r++) {
        const int i = t.i0 + r;
        const PRow r3 = prow(i + 2);
        float amC, fvC;  // row i+1
        pface32(V, i + 1, j, col_ok, r2, r3, qe(i + 1), amC, fvC);
        const int id = pidx(i, j, V.pit);
        if (col_ok && !(V.ifp && V.ifp[id])) {
            V.FH[id] = V.dpif * (fvB * amB + w3 * (fvC - fvA) * (amC - amA));
            if (step == 0) V.FL[id] = V.dpif * ((amB > 0.0f ? V.f[id - 1] : V.f[id]) * amB);
        }
        amA = amB;
        fvA = fvB;
        amB = amC;
        fvB = fvC;
        r2 = r3;
    }
}

}  // namespace vx
