// FP32 momentum moments (Rectangle::CalculateRhoAndJ, Rectangle.cpp:157-282) of the
// precision form: the device bodies, one coarse column per call, shared by the moments
// kernel (fields32.cu) and the persistent stage kernel (stage32.cu); both translation
// units are compiled with fused multiply-add allowed.
//
// The per-cell weights are evaluated in FP32 in a cancellation-free form; each lane keeps
// compensated (Kahan) FP32 sums, the lanes are combined as compensated FP32 pairs and the
// column sum is formed in FP64 by the assembly.  It does not reproduce the reference's
// rounding; the precision form states its error against the FP64 path instead.
#pragma once
#include <cuda_runtime.h>

#include "vx_kernels.hpp"

namespace vx {

using P32 = PatchT<float>;

// ---------------------------------------------------------------- moments
// One warp per coarse column i, all its finest sub-columns k at once.  Windows of 29
// outputs: lane l holds p index j = j0 - 1 + l; l_j needs G of the next lane, so lanes
// 0..30 have it and lanes 1..29 produce.
//   G_j = gamma_j + p_j = (1 + a) / (gamma_j - p_j)   (dimensionless, p in units of m c;
//         the second form where p_j < 0, free of cancellation),
//   dG  = G_{j+1} - G_j = dp (1 + (p_{j+1} + p_j) / (gamma_{j+1} + gamma_j)),
//   l_j = ln(G_{j+1} / G_j) = 2 atanh(z),  z = dG / (2 G_j + dG)
//       = 2 z (1 + z^2/3 + z^4/5 + z^6/7)  (Taylor series; for z <= 1/16 the next term
//         is below 3e-10 relative), ln(1 + u) otherwise,
//   rho_k += f_j,  J_k += f_j l_j + (1/48)(l_{j+1} - l_{j-1})(f_{j+1} - f_{j-1}).
constexpr int kMom32Out = 29;

// Compensated FP32 pair (value = hi + lo): TwoSum (Knuth) and FastTwoSum (Dekker)
// additions for the warp reduction of the lanes' Kahan sums.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ F2 f2_warp_sum(F2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        const F2 w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
        v = f2_add(v, w);
    }
    return v;
}

// l_j = ln(G_{j+1} / G_j) for a lane's p_j (see the table above); valid on lanes 0..30.
__device__ __forceinline__ float log_ratio32(float p, float pn, float g, float gn, float a, float dpn) {
    const float dG = dpn * (1.0f + __fdividef(pn + p, gn + g));
    const float G = p >= 0.0f ? g + p : __fdividef(1.0f + a, g - p);
    const float z = __fdividef(dG, 2.0f * G + dG);
    if (z <= 0.0625f) {
        const float z2 = z * z;
        return 2.0f * z * fmaf(z2, fmaf(z2, fmaf(z2, 1.0f / 7.0f, 0.2f), 1.0f / 3.0f), 1.0f);
    }
    // ln(1 + u) as logf(y) u / (y - 1), y = 1 + u rounded (Goldberg, "What every computer
    // scientist should know about floating-point arithmetic", 1991)
    const float u = __fdividef(dG, G);
    const float y1 = 1.0f + u;
    return logf(y1) * __fdividef(u, y1 - 1.0f);
}

__device__ __forceinline__ void kahan_add(float v, float &sum, float &comp) {
    const float y = v - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// Sub-columns k0 .. k0+KG-1 of coarse column i (rtb finest sub-columns): the f stencil
// and the interpolation's shared part are loaded and formed once per cell for the group.
// KG = 1 (rtb = 1) runs two windows per iteration to have two chains in flight; wider
// columns go through in groups of two, re-reading f from L1.
template <int KG>
__device__ __forceinline__ void moments_group(const P32 &P, const RunFields &F, int i, int k0, int lane) {
    constexpr int NW = KG == 1 ? 2 : 1;
    const unsigned full = 0xffffffffu;
    const int rtb = P.rtb;
    float a[KG], wk0[KG], wk1[KG], wk2[KG];
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int q = 0; q < KG; q++) {
        const int k = k0 + q;
        // cell-average A^2 at the finest cell (EMSolver::GetCellAverageASquared), made
        // dimensionless
        int xc = (i + P.x_pos) * rtb + k + F.pre;
        xc = xc > -1 ? xc : 0;
        xc = xc < F.nf ? xc : F.nf - 1;
        a[q] = P.a2nf * F.acell32[xc];
        wk0[q] = wk1[q] = wk2[q] = 0.0f;
        if (rtb > 1) {
            wk0[q] = P.relc32[3 * k];
            wk1[q] = P.relc32[3 * k + 1];
            wk2[q] = P.relc32[3 * k + 2];
        }
    }
    if (rtb > 1) {
        s0 = P.relc32[3 * rtb];
        s1 = P.relc32[3 * rtb + 1];
        s2 = P.relc32[3 * rtb + 2];
    }
    const float pmin = P.pminf, dpn = P.dpnf;
    const float c3 = 1.0f / 48.0f, inv_rtb = 1.0f / (float)rtb;  // rtb is a power of two
    const float *f = P.f1;
    const int pit = P.pitch;
    float chs[KG], chc[KG], cus[KG], cuc[KG];
#pragma unroll
    for (int q = 0; q < KG; q++) chs[q] = chc[q] = cus[q] = cuc[q] = 0.0f;
    for (int j0 = 0; j0 < P.np; j0 += NW * kMom32Out) {
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const int jw = j0 + w * kMom32Out;
            if (w > 0 && jw >= P.np) break;  // warp-uniform
            const int j = jw - 1 + lane;
            const float p = fmaf(dpn, (float)(j + P.p_pos), pmin);
            const float pn = fmaf(dpn, (float)(j + 1 + P.p_pos), pmin);
            // interpolation's shared part (Rectangle.cpp:139-155, 183-204)
            float f3 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f, fmean = 0.0f;
            if (j <= P.np) {
                f3 = f[pidx(i, j, pit)];
                if (rtb > 1) {
                    const float g1 = f[pidx(i - 2, j, pit)] - f3, g2 = f[pidx(i - 1, j, pit)] - f3;
                    const float g4 = f[pidx(i + 1, j, pit)] - f3, g5 = f[pidx(i + 2, j, pit)] - f3;
                    a1 = 0.104166666666667f * g1 - 0.708333333333334f * g2 + 0.708333333333334f * g4 - 0.104166666666667f * g5;
                    a2 = 0.117647058823529f * g1 + 0.029411764705882f * g2 + 0.029411764705882f * g4 + 0.117647058823529f * g5;
                    a3 = -0.083333333333333f * g1 + 0.166666666666667f * g2 - 0.166666666666667f * g4 + 0.083333333333334f * g5;
                    fmean = (s0 * a1 + s1 * a2 + s2 * a3) * inv_rtb + f3;
                }
            }
            const bool use = lane >= 1 && lane <= kMom32Out && j < P.np && !(P.nested && P.nested[pidx(i, j, pit)]);
#pragma unroll
            for (int q = 0; q < KG; q++) {
                const float s = 1.0f + p * p + a[q];
                const float g = s * rsqrtf(s);
                const float gn = __shfl_down_sync(full, g, 1);
                const float l = log_ratio32(p, pn, g, gn, a[q], dpn);
                const float V = rtb == 1 ? f3 : (wk0[q] * a1 + wk1[q] * a2 + wk2[q] * a3 + f3) + (f3 - fmean);
                const float lm = __shfl_up_sync(full, l, 1), lp = __shfl_down_sync(full, l, 1);
                const float Vm = __shfl_up_sync(full, V, 1), Vp = __shfl_down_sync(full, V, 1);
                kahan_add(use ? V : 0.0f, chs[q], chc[q]);
                kahan_add(use ? (V * l + c3 * (lp - lm) * (Vp - Vm)) : 0.0f, cus[q], cuc[q]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < KG; q++) {
        const F2 ch = f2_warp_sum(F2{chs[q], -chc[q]});
        const F2 cu = f2_warp_sum(F2{cus[q], -cuc[q]});
        if (lane == 0) {
            const int c = i * rtb + k0 + q;
            // the column sum as an FP32 pair in the column's double slot; k_assemble forms
            // the FP64 value and applies the scale (no FP64 instruction here)
            reinterpret_cast<float2 *>(P.chargeR)[c] = make_float2(ch.hi, ch.lo);
            reinterpret_cast<float2 *>(P.currentR)[c] = make_float2(cu.hi, cu.lo);
        }
    }
}

// One warp per coarse column (M.colidx holds i * rtb, the column's first finest
// sub-column).  No FP64 instruction: the A^2 of each sub-column comes from the FP32
// per-cell copy, the weights from the patch descriptor; the reduced pairs go to the
// assembly, which scales them in FP64.  All 32 lanes call it together.
__device__ __forceinline__ void moments32_column(const MomLaunch &M, int col, int lane) {
    const P32 &P = ((const P32 *)M.patches)[M.colpatch[col]];
    const int i = M.colidx[col] / P.rtb;
    const RunFields &F = M.fields[P.run];
    if (P.rtb == 1) moments_group<1>(P, F, i, 0, lane);
    else  // rtb is even (2, 4 or 8 in the FP32 form)
        for (int k0 = 0; k0 < P.rtb; k0 += 2) moments_group<2>(P, F, i, k0, lane);
}

// Element e of the FP32 copy of a^2 that a stage's face kernels read (runs of
// M.maxnf + 1 entries each; the Maxwell stage, which rewrites a^2, starts only after the
// moments).
__device__ __forceinline__ void asq32_copy(const MomLaunch &M, int e) {
    const int per = M.maxnf + 1;
    const RunFields &F = M.fields[e / per];
    const int x = e % per;
    if (x <= F.n) F.asq32[x] = (float)F.asq[x];
}

// FP32 copy of Ay^2 + Az^2 (slot 1) at cell x of a run's field grid, read by the moments;
// unfused, as the Maxwell update forms the same copy.
__device__ __forceinline__ void acell32_cell(const RunFields *fields, int run, int x) {
    const RunFields &F = fields[run];
    if (x >= F.nf) return;
    const double ay = F.Ay[F.nf + x], az = F.Az[F.nf + x];
    F.acell32[x] = (float)__dadd_rn(__dmul_rn(ay, ay), __dmul_rn(az, az));
}

}  // namespace vx
