// Field-side kernels of the FP32 precision form.
//
//  * k32_moments — momentum moments (Rectangle::CalculateRhoAndJ, Rectangle.cpp:157-282)
//    of FP32 (scaled) f: the per-cell weights are evaluated in FP32 in a cancellation-free
//    form; each lane keeps compensated (Kahan) FP32 sums and the lanes are combined in
//    FP64.
//  * k_poisson_fast — the Poisson solve (EMFieldSolver::UpdatePotential,
//    EMSolver.cpp:156-192) in FP64 by an O(n) scan algorithm instead of the dense LU.
//
// Neither kernel reproduces the reference's rounding; the precision form states its
// error against the FP64 path instead.
#include <cuda_runtime.h>
#include "vx_kernels.hpp"

namespace vx {

using P32 = PatchT<float>;

// ---------------------------------------------------------------- moments
// One warp per moment column (coarse column i, finest sub-column k).  Windows of 29
// outputs: lane l holds p index j = j0 - 1 + l; l_j needs G of the next lane, so lanes
// 0..30 have it and lanes 1..29 produce.
//   G_j = gamma_j + p_j (dimensionless, p in units of m c),
//   l_j = ln(G_{j+1} / G_j) = log1p(dG / G_j),
//   dG  = dp (1 + (p_{j+1} + p_j) / (gamma_{j+1} + gamma_j))   (no cancellation),
//   rho_k += f_j,  J_k += f_j l_j + (1/48)(l_{j+1} - l_{j-1})(f_{j+1} - f_{j-1}).
constexpr int kMom32Out = 29;

__device__ __forceinline__ float rel_value32(const P32 &P, const float *f, int i, int j, int k, const float *w) {
    const int pit = P.pitch;
    const float f3 = f[pidx(i, j, pit)];
    if (P.rtb == 1) return f3;
    const float g1 = f[pidx(i - 2, j, pit)] - f3, g2 = f[pidx(i - 1, j, pit)] - f3;
    const float g4 = f[pidx(i + 1, j, pit)] - f3, g5 = f[pidx(i + 2, j, pit)] - f3;
    const float a1 = 0.104166666666667f * g1 - 0.708333333333334f * g2 + 0.708333333333334f * g4 - 0.104166666666667f * g5;
    const float a2 = 0.117647058823529f * g1 + 0.029411764705882f * g2 + 0.029411764705882f * g4 + 0.117647058823529f * g5;
    const float a3 = -0.083333333333333f * g1 + 0.166666666666667f * g2 - 0.166666666666667f * g4 + 0.083333333333334f * g5;
    float te = 0.0f, mine = 0.0f;
    for (int q = 0; q < P.rtb; q++) {
        const float v = w[3 * q] * a1 + w[3 * q + 1] * a2 + w[3 * q + 2] * a3 + f3;
        te += v;
        if (q == k) mine = v;
    }
    return mine + (f3 - te / (float)P.rtb);
}

__global__ void k32_moments(MomLaunch M) {
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
    const double ay = F.Ay[F.nf + xc], az = F.Az[F.nf + xc];
    const float a = (float)(P.qq * ((ay * ay) + (az * az)) * P.g2);
    float w[24];
    for (int q = 0; q < 3 * P.rtb && q < 24; q++) w[q] = (float)P.relc[q];
    const float pmin = P.pminf, dpn = P.dpnf;
    const float c3 = 1.0f / 48.0f;
    const float *f = P.f1;
    const unsigned full = 0xffffffffu;
    // per-lane compensated FP32 sums (Kahan); FP64 only for the final warp reduction
    float chs = 0.0f, chc = 0.0f, cus = 0.0f, cuc = 0.0f;
    for (int j0 = 0; j0 < P.np; j0 += kMom32Out) {
        const int j = j0 - 1 + lane;
        const float p = fmaf(dpn, (float)(j + P.p_pos), pmin);
        const float g = sqrtf(1.0f + p * p + a);
        const float gn = __shfl_down_sync(full, g, 1);
        const float pn = __shfl_down_sync(full, p, 1);
        const float dG = dpn * (1.0f + (pn + p) / (gn + g));
        const float l = log1pf(dG / (g + p));  // valid on lanes 0..30
        float V = 0.0f;
        if (j <= P.np) V = rel_value32(P, f, i, j, k, w);
        const float lm = __shfl_up_sync(full, l, 1), lp = __shfl_down_sync(full, l, 1);
        const float Vm = __shfl_up_sync(full, V, 1), Vp = __shfl_down_sync(full, V, 1);
        const bool use = lane >= 1 && lane <= kMom32Out && j < P.np && !(P.nested && P.nested[pidx(i, j, P.pitch)]);
        if (use) {
            float y = V - chc;
            float t = chs + y;
            chc = (t - chs) - y;
            chs = t;
            y = (V * l + c3 * (lp - lm) * (Vp - Vm)) - cuc;
            t = cus + y;
            cuc = (t - cus) - y;
            cus = t;
        }
    }
    double ch = (double)chs - (double)chc, cu = (double)cus - (double)cuc;
    for (int o = 16; o > 0; o >>= 1) {
        ch += __shfl_down_sync(full, ch, o);
        cu += __shfl_down_sync(full, cu, o);
    }
    if (lane == 0) {
        const double q = P.q;
        const double c2 = 1.0 / ((1.0 / P.mass) * kCInv);  // m c, the reference's c2
        const double inv = 1.0 / P.fnorm;
        P.chargeR[c] = ch * inv * (P.dp * q);
        P.currentR[c] = cu * inv * c2 * (-q * q / P.mass);
    }
}

void launch_moments32(const MomLaunch &M) {
    if (M.ncols == 0) return;
    const int threads = 256;
    const int blocks = (M.ncols * 32 + threads - 1) / threads;
    k32_moments<<<blocks, threads, 0, M.stream>>>(M);
}

// ---------------------------------------------------------------- fast Poisson
// The LU solve sees M = P^T, P the reference's row-major stencil matrix (EMSolver.cpp:
// 41-67).  Column 0 of M is e_0, so M = [[1, r^T], [0, B]]: phi[1:] = B^{-1} b[1:] and
// phi_0 = b_0 - (w1 phi_1 + w2 phi_2 + w2 phi_{n-2} + w1 phi_{n-1}).  B (m = n-1) is the
// pentadiagonal Toeplitz stencil T = (w2, w1, w3, w1, w2) plus the corner pair
// w2 (e_0 e_{m-1}^T + e_{m-1} e_0^T).  The stencil's symbol has the roots 1, 1, rho, 1/rho
// (rho = 7 - 4 sqrt 3), so T = c G G^T + (a 2x2 block at the top left) with
// G = (I - S)(I - rho S), c = w2 / rho.  Hence
//   B^{-1} v = z - Y K (z_0, z_1, z_{m-1}),   z = (1/c) G^{-T} G^{-1} v,
// with Y = (1/c) G^{-T} G^{-1} [e_0 e_1 e_{m-1}] and the 3x3 K precomputed on the host
// (Woodbury).  G^{-1} and G^{-T} are two prefix sums (block scans) and two decaying
// first-order recurrences (segment-local with a short carry gather).
constexpr int kPfThreads = 1024;

// Exclusive block scan of sums (prefix sums of one value per thread).
__device__ double block_exclusive_sum(double v, double *sb) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned full = 0xffffffffu;
    double x = v;
    for (int o = 1; o < 32; o <<= 1) {
        double p = __shfl_up_sync(full, x, o);
        if (lane >= o) x += p;
    }
    if (lane == 31) sb[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double w = (lane < (int)(blockDim.x >> 5)) ? sb[lane] : 0.0;
        for (int o = 1; o < 32; o <<= 1) {
            double p = __shfl_up_sync(full, w, o);
            if (lane >= o) w += p;
        }
        sb[lane] = w;
    }
    __syncthreads();
    double ex = x - v;
    if (wid > 0) ex += sb[wid - 1];
    __syncthreads();
    return ex;
}

// y_k = v_k + mult * y_{k-1} over v[0..m) in scan order (reversed when REV), in place.
// mult = 1: prefix sums.  mult = rho (< 0.072): the carry into a segment is
// sum_q rho^{(q-1)L} y_end(segment - q), and rho^{qL} drops below 1e-20 after a few
// segments (three for L >= 8), so a short gather replaces the scan.
template <bool REV>
__device__ void recurrence_pass(double *v, int m, double mult, const double *powtab, double *sa, double *sb) {
    const int T = blockDim.x;
    const int L = (m + T - 1) / T;
    const int k0 = threadIdx.x * L, k1 = min(m, k0 + L);
    double y = 0.0;
    for (int k = k0; k < k1; k++) {
        const int idx = REV ? m - 1 - k : k;
        y = v[idx] + mult * y;
        v[idx] = y;
    }
    double carry;
    if (mult == 1.0) {
        carry = block_exclusive_sum(y, sb);
    } else {
        sa[threadIdx.x] = y;  // segment end without carry (sa holds blockDim doubles)
        __syncthreads();
        const int t = threadIdx.x;
        const double aL = powtab[L - 1];  // mult^L
        carry = 0.0;
        double wgt = 1.0;
        for (int q = 1; q <= t && wgt > 1e-20; q++) {
            carry += wgt * sa[t - q];
            wgt *= aL;
        }
        __syncthreads();
    }
    for (int k = k0; k < k1; k++) {
        const int idx = REV ? m - 1 - k : k;
        v[idx] += powtab[k - k0] * carry;  // mult^(k-k0+1)
    }
    __syncthreads();
}

__device__ __forceinline__ double efield_fast(const double *phi, int n, double fcoef, double ex0, int i) {
    int ip1 = i + 1, im1 = i - 1, ip2 = i + 2, im2 = i - 2;
    ip1 = (ip1 > -1) ? ip1 : (ip1 + n);
    im1 = (im1 > -1) ? im1 : (im1 + n);
    ip2 = (ip2 > -1) ? ip2 : (ip2 + n);
    im2 = (im2 > -1) ? im2 : (im2 + n);
    ip1 = (ip1 < n) ? ip1 : (ip1 - n);
    im1 = (im1 < n) ? im1 : (im1 - n);
    ip2 = (ip2 < n) ? ip2 : (ip2 - n);
    im2 = (im2 < n) ? im2 : (im2 - n);
    return -fcoef * (8 * (phi[ip1] - phi[im1]) - phi[ip2] + phi[im2]) + ex0;
}

__global__ void __launch_bounds__(kPfThreads) k_poisson_fast(PoissonFastLaunch L) {
    __shared__ double sa[kPfThreads], sb[32];
    __shared__ double pw_one[kPfMaxSeg], pw_rho[kPfMaxSeg];
    __shared__ double tvec[3];
    const int run = blockIdx.x;
    RunFields &F = L.fields[run];
    const PoissonFastDev &D = L.pf[run];
    const int n = F.n, m = n - 1;
    double *b = F.efin;     // right-hand side (scratch until E_x is recomputed)
    double *x = F.phi + 1;  // phi[1..n-1] is the working vector
    const double te = kEps0Inv, w = L.w[run];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double v = te * (F.charge[i] + F.neut[i]);
        b[i] = v * w;
    }
    for (int q = threadIdx.x; q < kPfMaxSeg; q += blockDim.x) {
        pw_one[q] = 1.0;
        pw_rho[q] = pow(D.rho, (double)(q + 1));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x) x[k] = b[k + 1];
    __syncthreads();
    recurrence_pass<false>(x, m, 1.0, pw_one, sa, sb);    // (I - S)^{-1}
    recurrence_pass<false>(x, m, D.rho, pw_rho, sa, sb);  // (I - rho S)^{-1}
    recurrence_pass<true>(x, m, D.rho, pw_rho, sa, sb);   // (I - rho S^T)^{-1}
    recurrence_pass<true>(x, m, 1.0, pw_one, sa, sb);     // (I - S^T)^{-1}
    for (int k = threadIdx.x; k < m; k += blockDim.x) x[k] *= D.c_inv;
    __syncthreads();
    if (threadIdx.x == 0) {
        const double u0 = x[0], u1 = x[1], u2 = x[m - 1];
        for (int r = 0; r < 3; r++) tvec[r] = D.K[3 * r] * u0 + D.K[3 * r + 1] * u1 + D.K[3 * r + 2] * u2;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += blockDim.x)
        x[k] -= D.Y[3 * k] * tvec[0] + D.Y[3 * k + 1] * tvec[1] + D.Y[3 * k + 2] * tvec[2];
    __syncthreads();
    double *phi = F.phi;
    if (threadIdx.x == 0) {
        phi[0] = b[0] - (D.w1 * phi[1] + D.w2 * phi[2] + D.w2 * phi[n - 2] + D.w1 * phi[n - 1]);
        const double ex0 = *F.ex0;
        const double e_m1 = efield_fast(phi, n, L.fcoef[run], ex0, -1);
        const double e_0 = efield_fast(phi, n, L.fcoef[run], ex0, 0);
        *F.ex0 = ex0 + -(e_m1 + e_0) * 0.5;
    }
    __syncthreads();
    const double ex0 = *F.ex0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) F.efin[i] = efield_fast(phi, n, L.fcoef[run], ex0, i);
}

__global__ void k_fields_to_f32(RunFields *fields, int nruns, int which) {
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
    k_fields_to_f32<<<g, 256, 0, s>>>(fields, nruns, which);
}

void launch_poisson_fast(const PoissonFastLaunch &L) {
    if (L.nruns == 0) return;
    k_poisson_fast<<<L.nruns, kPfThreads, 0, L.stream>>>(L);
}

}  // namespace vx
