// O(n) Poisson solve by prefix scans (EMFieldSolver::UpdatePotential,
// EMSolver.cpp:156-192): used by the FP32 precision form and, on request, by FP64 runs.
//
// The reference's LU solve sees M = P^T, P its row-major stencil matrix (EMSolver.cpp:
// 41-67).  Column 0 of M is e_0, so M = [[1, r^T], [0, B]]: phi[1:] = B^{-1} b[1:] and
// phi_0 = b_0 - (w1 phi_1 + w2 phi_2 + w2 phi_{n-2} + w1 phi_{n-1}).  B (m = n-1) is the
// pentadiagonal Toeplitz stencil T = (w2, w1, w3, w1, w2) plus the corner pair
// w2 (e_0 e_{m-1}^T + e_{m-1} e_0^T).  The stencil's symbol has the roots 1, 1, rho, 1/rho
// (rho = 7 - 4 sqrt 3), so T = c G G^T + (a 2x2 block at the top left) with
// G = (I - S)(I - rho S), c = w2 / rho.  Hence
//   B^{-1} v = z - Y K (z_0, z_1, z_{m-1}),   z = (1/c) G^{-T} G^{-1} v,
// with Y = (1/c) G^{-T} G^{-1} [e_0 e_1 e_{m-1}] and the 3x3 K precomputed on the host
// (Woodbury, poisson_fast.cpp).  G^{-1} and G^{-T} are two prefix sums and two decaying
// first-order recurrences.
//
// One thread-block cluster per run: the kPsCluster blocks of a cluster hold consecutive
// chunks of the vector in shared memory (T segments of L elements each, stored
// segment-minor so that a warp's threads walk their segments on different banks).  A
// pass runs every segment serially, then fixes the segments up with their carry: the
// prefix sum of the preceding segment sums (a block scan plus the preceding blocks' totals
// read through distributed shared memory), or for the decaying recurrences the sum over
// preceding segment ends weighted by rho^{L (q-1)}, which drops below 1e-20 after a few
// segments (three for L >= 8, which the block size is chosen for).  The cluster barriers
// are hardware barriers of co-scheduled blocks.
//
// FP64 throughout, with fused multiply-adds (E_x itself comes from k_efield, which keeps
// the reference's rounding).  The result is not the LU's rounding order; both have the
// error the discrete system's conditioning (~n^2) allows, about 1e-11 relative at
// n = 2048 and 1e-9 at n = 8192 against the exact solution.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "vx_kernels.hpp"

namespace vx {

namespace {

namespace cg = cooperative_groups;

constexpr int kPsMaxTerms = 24;  // carry-gather terms of a decaying pass (rho^24 < 1e-27)

// E_x at cell i (EMSolver::GetEfield order); phi read past L1, since other blocks of the
// cluster wrote it in this launch.
__device__ __forceinline__ double efield_at(const double *phi, int n, double fcoef, double ex0, int i) {
    int ip1 = i + 1, im1 = i - 1, ip2 = i + 2, im2 = i - 2;
    ip1 = (ip1 > -1) ? ip1 : (ip1 + n);
    im1 = (im1 > -1) ? im1 : (im1 + n);
    ip2 = (ip2 > -1) ? ip2 : (ip2 + n);
    im2 = (im2 > -1) ? im2 : (im2 + n);
    ip1 = (ip1 < n) ? ip1 : (ip1 - n);
    im1 = (im1 < n) ? im1 : (im1 - n);
    ip2 = (ip2 < n) ? ip2 : (ip2 - n);
    im2 = (im2 < n) ? im2 : (im2 - n);
    return -fcoef * (8 * (__ldcg(phi + ip1) - __ldcg(phi + im1)) - __ldcg(phi + ip2) + __ldcg(phi + im2)) + ex0;
}

// Exclusive scan of one value per thread, in thread order; the block's total goes to *tot.
__device__ double block_exclusive_sum(double v, double *sb, double *tot) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    double x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const double p = __shfl_up_sync(full, x, o);
        if (lane >= o) x = x + p;
    }
    if (lane == 31) sb[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double w = (lane < nw) ? sb[lane] : 0.0;
        for (int o = 1; o < 32; o <<= 1) {
            const double p = __shfl_up_sync(full, w, o);
            if (lane >= o) w = w + p;
        }
        sb[lane] = w;
        if (lane == nw - 1) *tot = w;
    }
    __syncthreads();
    double ex = __shfl_up_sync(full, x, 1);
    if (lane == 0) ex = 0.0;
    if (wid > 0) ex = sb[wid - 1] + ex;
    return ex;
}

// Per-block scratch of a pass.
struct ScanScratch {
    double *sa;     // [T] segment ends without carry (read across the cluster)
    double *sb;     // [32] warp totals
    double *pw;     // [L] mult^(s+1) of the decaying passes
    double *wt;     // [kPsMaxTerms] rho^(L q) carry weights
    double *s_tot;  // block total of a prefix-sum pass (read across the cluster)
    double *s_pre;  // preceding blocks' totals
    int nterms;     // carry terms of a decaying pass
};

// y_k = v_k + mult y_{k-1} over the run's m unknowns, in place, ascending (or descending
// when REV); mult = 1 when UNIT.  Thread t owns segment t (REV: segment T-1-t, so thread
// order is scan order either way); blocks are in scan order by rank (REV: reversed).
// Segments past the end of the vector are short or empty; in scan order they come last
// (REV: first), so no full-length weight ever crosses one.
template <bool REV, bool UNIT>
__device__ void scan_pass(cg::cluster_group &cl, double *xs, int L, int m, int g0, double mult, const ScanScratch &W) {
    constexpr int C = kPsCluster;
    const int T = blockDim.x, stride = T + 1;
    const int rank = (int)cl.block_rank();
    const int tid = threadIdx.x;
    const int seg = REV ? T - 1 - tid : tid;
    const int len = max(0, min(L, m - (g0 + seg * L)));
    double y = 0.0;
    for (int s = 0; s < len; s++) {
        double *p = &xs[(REV ? len - 1 - s : s) * stride + seg];
        y = UNIT ? (*p + y) : (*p + mult * y);
        *p = y;
    }
    const int cpos = REV ? C - 1 - rank : rank;  // this block's place in scan order
    double carry;
    if (UNIT) {
        const double ex = block_exclusive_sum(y, W.sb, W.s_tot);
        cl.sync();
        if (tid == 0) {
            double pre = 0.0;
            for (int q = 0; q < cpos; q++) pre = pre + *cl.map_shared_rank(W.s_tot, REV ? C - 1 - q : q);
            *W.s_pre = pre;
        }
        __syncthreads();
        carry = *W.s_pre + ex;
    } else {
        W.sa[tid] = y;
        cl.sync();
        // carry = sum_q rho^{L (q-1)} y_end(sp - q): terms below 1e-20 relative are dropped
        const int sp = cpos * T + tid;
        const int nq = min(W.nterms, sp);
        carry = 0.0;
        for (int q = 1; q <= nq; q++) {
            const int src = sp - q;
            const int r = REV ? C - 1 - src / T : src / T;
            carry = carry + W.wt[q - 1] * cl.map_shared_rank(W.sa, r)[src % T];
        }
    }
    cl.sync();  // every remote read of sa / s_tot is done before the next pass rewrites them
    for (int s = 0; s < len; s++) {
        double *p = &xs[(REV ? len - 1 - s : s) * stride + seg];
        *p = *p + (UNIT ? carry : W.pw[s] * carry);
    }
    __syncthreads();
}

__global__ void __cluster_dims__(kPsCluster, 1, 1) __launch_bounds__(kPsMaxThreads)
    k_poisson_scan(PoissonFastLaunch P) {
    VX_PDL_WAIT();
    extern __shared__ double xs[];  // [L][T + 1]: element (segment s, offset o) at o (T + 1) + s
    __shared__ double sa[kPsMaxThreads], sb[32], pw[kPsMaxSeg], wt[kPsMaxTerms], s_tot, s_pre, s_u[3];
    __shared__ int s_nterms;
    cg::cluster_group cl = cg::this_cluster();
    const int T = blockDim.x, stride = T + 1;
    const int run = blockIdx.x / kPsCluster;
    const int rank = (int)cl.block_rank();
    RunFields &F = P.fields[run];
    const PoissonFastDev &D = P.pf[run];
    const int n = F.n, m = n - 1;
    const int L = (m + T * kPsCluster - 1) / (T * kPsCluster);
    const int g0 = rank * T * L;  // first unknown of this block's chunk
    // right-hand side (dx^2 / eps0) (rho + rho_neutral), x_k = b_{k+1}
    const double te = kEps0Inv, w = P.w[run];
    for (int l = threadIdx.x; l < T * L; l += T) {
        const int g = g0 + l;
        double v = 0.0;
        if (g < m) {
            const double r = te * (F.charge[g + 1] + F.neut[g + 1]);
            v = r * w;
        }
        xs[(l % L) * stride + l / L] = v;
    }
    if (threadIdx.x == 0) {  // powers by repeated products (a library pow is a long FP64 chain here)
        double x = D.rho;
        for (int q = 0; q < L; q++) {
            pw[q] = x;
            x = x * D.rho;
        }
        const double aL = pw[L - 1];
        x = 1.0;
        int q = 0;
        while (q < kPsMaxTerms && x > 1e-20) {
            wt[q++] = x;
            x = x * aL;
        }
        s_nterms = q;
    }
    __syncthreads();
    const ScanScratch W{sa, sb, pw, wt, &s_tot, &s_pre, s_nterms};
    scan_pass<false, true>(cl, xs, L, m, g0, 1.0, W);    // (I - S)^{-1}
    scan_pass<false, false>(cl, xs, L, m, g0, D.rho, W);  // (I - rho S)^{-1}
    scan_pass<true, false>(cl, xs, L, m, g0, D.rho, W);   // (I - rho S^T)^{-1}
    scan_pass<true, true>(cl, xs, L, m, g0, 1.0, W);     // (I - S^T)^{-1}
    cl.sync();  // every chunk final before the Woodbury entries are read across blocks
    if (threadIdx.x < 3) {
        const int g = threadIdx.x == 2 ? m - 1 : threadIdx.x;
        const int r = g / (T * L), l = g - r * T * L;
        s_u[threadIdx.x] = cl.map_shared_rank(xs, r)[(l % L) * stride + l / L] * D.c_inv;
    }
    __syncthreads();
    double t[3];
    for (int r = 0; r < 3; r++) t[r] = D.K[3 * r] * s_u[0] + D.K[3 * r + 1] * s_u[1] + D.K[3 * r + 2] * s_u[2];
    for (int l = threadIdx.x; l < T * L; l += T) {
        const int g = g0 + l;
        if (g >= m) break;
        const double z = xs[(l % L) * stride + l / L] * D.c_inv;
        F.phi[g + 1] = z - (D.Y[3 * g] * t[0] + D.Y[3 * g + 1] * t[1] + D.Y[3 * g + 2] * t[2]);
    }
    __threadfence();
    cl.sync();  // phi[1..n-1] written; no block touches another's shared memory after this
    if (rank == 0 && threadIdx.x == 0) {
        double *phi = F.phi;
        const double r0 = te * (F.charge[0] + F.neut[0]);
        phi[0] = r0 * w - (D.w1 * __ldcg(phi + 1) + D.w2 * __ldcg(phi + 2) + D.w2 * __ldcg(phi + n - 2) +
                           D.w1 * __ldcg(phi + n - 1));
        __threadfence_block();
        const double ex0 = *F.ex0;
        const double e_m1 = efield_at(phi, n, P.fcoef[run], ex0, -1);
        const double e_0 = efield_at(phi, n, P.fcoef[run], ex0, 0);
        *F.ex0 = ex0 + -(e_m1 + e_0) * 0.5;
        __threadfence();
    }
    cl.sync();  // phi[0] and the new Ex0 are visible to every block of the cluster
    // E_x on the finest grid (EMFieldSolver::GetEfield), each block a contiguous share
    const double ex0 = __ldcg(F.ex0), fc = P.fcoef[run];
    const int share = (n + kPsCluster - 1) / kPsCluster;
    const int i1 = min(n, (rank + 1) * share);
    for (int i = rank * share + threadIdx.x; i < i1; i += T) {
        const double e = efield_at(F.phi, n, fc, ex0, i);
        F.efin[i] = e;
        if (P.f32) F.efin32[i] = (float)e;
    }
}

// Threads per block: segments of about 8 elements (a decaying pass then gathers three
// carry terms), 32 to kPsMaxThreads threads.
int scan_threads(int maxn) {
    const int m = maxn - 1;
    int t = 32;
    while (t < kPsMaxThreads && (long long)t * kPsCluster * 8 < m) t *= 2;
    return t;
}

}  // namespace

size_t poisson_scan_smem(int maxn) {
    const int m = maxn - 1, T = scan_threads(maxn);
    const int L = (m + T * kPsCluster - 1) / (T * kPsCluster);
    return (size_t)L * (T + 1) * sizeof(double);
}

void launch_poisson_fast(const PoissonFastLaunch &L) {
    if (L.nruns == 0) return;
    const size_t smem = poisson_scan_smem(L.maxn);
    cudaFuncSetAttribute(k_poisson_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    vx_launch(k_poisson_scan, L.nruns * kPsCluster, scan_threads(L.maxn), smem, L.stream, L);
}

}  // namespace vx
