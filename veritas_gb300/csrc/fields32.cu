// Field-side kernels of the FP32 precision form.
//
//  * k32_moments — momentum moments (Rectangle::CalculateRhoAndJ, Rectangle.cpp:157-282)
//    of FP32 (scaled) f: the per-cell weights are evaluated in FP32 in a cancellation-free
//    form; each lane keeps compensated (Kahan) FP32 sums, the lanes are combined as
//    compensated FP32 pairs and the column sum is formed in FP64.
//
// It does not reproduce the reference's rounding; the precision form states its error
// against the FP64 path instead.
#include <cuda_runtime.h>
#include "vx_kernels.hpp"

namespace vx {

using P32 = PatchT<float>;

// ---------------------------------------------------------------- moments
// One warp per moment column (coarse column i, finest sub-column k).  Windows of 29
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

// Interpolated value on finest sub-cell k of coarse cell (i, j) (Rectangle.cpp:139-155,
// 183-204): wk = weights of sub-cell k, ws = the weights summed over all sub-cells, so
// the conservative correction needs no loop over the sub-cells.
struct RelWeights {
    float k0, k1, k2, s0, s1, s2;
};

__device__ __forceinline__ float rel_value32(const P32 &P, const float *f, int i, int j, const RelWeights &w,
                                             float inv_rtb) {
    const int pit = P.pitch;
    const float f3 = f[pidx(i, j, pit)];
    if (P.rtb == 1) return f3;
    const float g1 = f[pidx(i - 2, j, pit)] - f3, g2 = f[pidx(i - 1, j, pit)] - f3;
    const float g4 = f[pidx(i + 1, j, pit)] - f3, g5 = f[pidx(i + 2, j, pit)] - f3;
    const float a1 = 0.104166666666667f * g1 - 0.708333333333334f * g2 + 0.708333333333334f * g4 - 0.104166666666667f * g5;
    const float a2 = 0.117647058823529f * g1 + 0.029411764705882f * g2 + 0.029411764705882f * g4 + 0.117647058823529f * g5;
    const float a3 = -0.083333333333333f * g1 + 0.166666666666667f * g2 - 0.166666666666667f * g4 + 0.083333333333334f * g5;
    const float mine = w.k0 * a1 + w.k1 * a2 + w.k2 * a3 + f3;
    const float mean = (w.s0 * a1 + w.s1 * a2 + w.s2 * a3) * inv_rtb + f3;
    return mine + (f3 - mean);
}

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

// No FP64 instruction per cell or per lane: the A^2 of the column comes from the FP32
// per-cell copy, the weights and the final scales from the patch descriptor; one lane
// converts the two reduced pairs to FP64.
__global__ void k32_moments(MomLaunch M) {
    VX_PDL_WAIT();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= M.ncols) return;
    const P32 &P = ((const P32 *)M.patches)[M.colpatch[warp]];
    const int c = M.colidx[warp];
    const int i = c / P.rtb, k = c - i * P.rtb;
    const RunFields &F = M.fields[P.run];
    // cell-average A^2 at the finest cell (EMSolver::GetCellAverageASquared), made
    // dimensionless
    int xc = (i + P.x_pos) * P.rtb + k + F.pre;
    xc = xc > -1 ? xc : 0;
    xc = xc < F.nf ? xc : F.nf - 1;
    const float a = P.a2nf * F.acell32[xc];
    RelWeights w{0, 0, 0, 0, 0, 0};
    float inv_rtb = 1.0f;
    if (P.rtb > 1) {
        const float *rw = P.relc32;
        w = {rw[3 * k], rw[3 * k + 1], rw[3 * k + 2], rw[3 * P.rtb], rw[3 * P.rtb + 1], rw[3 * P.rtb + 2]};
        inv_rtb = 1.0f / (float)P.rtb;
    }
    const float pmin = P.pminf, dpn = P.dpnf;
    const float c3 = 1.0f / 48.0f;
    const float *f = P.f1;
    const unsigned full = 0xffffffffu;
    // per-lane compensated FP32 sums (Kahan)
    float chs = 0.0f, chc = 0.0f, cus = 0.0f, cuc = 0.0f;
    auto kahan = [](float v, float &sum, float &comp) {
        float y = v - comp;
        float t = sum + y;
        comp = (t - sum) - y;
        sum = t;
    };
    // contributions of the window starting at p index j0 (zero on lanes that produce
    // nothing); warp-uniform, so two windows can be in flight per iteration
    auto window = [&](int j0, float &vc, float &vj) {
        const int j = j0 - 1 + lane;
        const float p = fmaf(dpn, (float)(j + P.p_pos), pmin);
        const float g = (1.0f + p * p + a) * rsqrtf(1.0f + p * p + a);
        const float gn = __shfl_down_sync(full, g, 1);
        const float pn = __shfl_down_sync(full, p, 1);
        const float dG = dpn * (1.0f + __fdividef(pn + p, gn + g));
        const float G = p >= 0.0f ? g + p : __fdividef(1.0f + a, g - p);
        const float z = __fdividef(dG, 2.0f * G + dG);
        float l;  // valid on lanes 0..30
        if (z <= 0.0625f) {
            const float z2 = z * z;
            l = 2.0f * z * fmaf(z2, fmaf(z2, fmaf(z2, 1.0f / 7.0f, 0.2f), 1.0f / 3.0f), 1.0f);
        } else {
            // ln(1 + u) as logf(y) u / (y - 1), y = 1 + u rounded (Goldberg, "What every
            // computer scientist should know about floating-point arithmetic", 1991)
            const float u = __fdividef(dG, G);
            const float y1 = 1.0f + u;
            l = logf(y1) * __fdividef(u, y1 - 1.0f);
        }
        float V = 0.0f;
        if (j <= P.np) V = rel_value32(P, f, i, j, w, inv_rtb);
        const float lm = __shfl_up_sync(full, l, 1), lp = __shfl_down_sync(full, l, 1);
        const float Vm = __shfl_up_sync(full, V, 1), Vp = __shfl_down_sync(full, V, 1);
        const bool use = lane >= 1 && lane <= kMom32Out && j < P.np && !(P.nested && P.nested[pidx(i, j, P.pitch)]);
        vc = use ? V : 0.0f;
        vj = use ? (V * l + c3 * (lp - lm) * (Vp - Vm)) : 0.0f;
    };
    for (int j0 = 0; j0 < P.np; j0 += 2 * kMom32Out) {
        float c0, j0v, c1 = 0.0f, j1v = 0.0f;
        window(j0, c0, j0v);
        if (j0 + kMom32Out < P.np) window(j0 + kMom32Out, c1, j1v);
        kahan(c0, chs, chc);
        kahan(j0v, cus, cuc);
        kahan(c1, chs, chc);
        kahan(j1v, cus, cuc);
    }
    const F2 ch = f2_warp_sum(F2{chs, -chc});
    const F2 cu = f2_warp_sum(F2{cus, -cuc});
    if (lane == 0) {
        P.chargeR[c] = ((double)ch.hi + (double)ch.lo) * P.msc_rho;
        P.currentR[c] = ((double)cu.hi + (double)cu.lo) * P.msc_j;
    }
}

// FP32 copy of Ay^2 + Az^2 (slot 1) over every run's field grid, read by k32_moments.
__global__ void k_acell32(const RunFields *fields, int nruns) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= nruns) return;
    const RunFields &F = fields[run];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= F.nf) return;
    const double ay = F.Ay[F.nf + x], az = F.Az[F.nf + x];
    F.acell32[x] = (float)((ay * ay) + (az * az));
}

void launch_moments32(const MomLaunch &M) {
    if (M.ncols == 0) return;
    vx_launch(k_acell32, dim3((M.maxnf + 255) / 256, M.nruns), 256, 0, M.stream, M.fields, M.nruns);
    const int threads = 256;
    const int blocks = (M.ncols * 32 + threads - 1) / threads;
    vx_launch(k32_moments, blocks, threads, 0, M.stream, M);
}

__global__ void k_fields_to_f32(RunFields *fields, int nruns, int which) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= nruns) return;
    RunFields &F = fields[run];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if ((which & 1) && x <= F.n) F.asq32[x] = (float)F.asq[x];
    if ((which & 2) && x < F.n) F.efin32[x] = (float)F.efin[x];
}

void launch_fields_to_f32(RunFields *fields, int nruns, int maxn, int which, cudaStream_t s) {
    if (nruns == 0) return;
    dim3 g((maxn + 1 + 255) / 256, nruns);
    vx_launch(k_fields_to_f32, g, 256, 0, s, fields, nruns, which);
}

}  // namespace vx
