// FP64 field-side kernels: momentum moments (Rectangle::CalculateRhoAndJ, MKL path
// Rectangle.cpp:157-237), finest-grid assembly (Level.cpp:19-62, EMSolver.cpp:104-122),
// Poisson solve with the precomputed LU factors (EMSolver.cpp:156-192), the transverse
// Maxwell RK stage with face interpolation of A (EMSolver.cpp:194-619) and the CFL bound
// (EMSolver.cpp:631-664).
//
// Compiled with --fmad=false so each double expression keeps the reference's operations
// and evaluation order.
#include <cuda_runtime.h>
#include <algorithm>
#include "fast64.cuh"
#include "field_ops.cuh"
#include "vx_kernels.hpp"

namespace vx {

using P64 = PatchT<double>;

// Interpolated value of f on the finest sub-cells of coarse cell (i, j), rtb > 1, with the
// conservative correction (Rectangle.cpp:139-155 and :183-204; the reference's fixed
// 12-entry interpolation matrix, Rectangle.cpp:76-89).  rel_shared forms what all
// sub-cells share — f3, the interpolation coefficients, the correction cor from the sum
// over every sub-cell's value — and sub-cell k's value is rel_pick(k) + cor, in the
// reference's operations and order.
__device__ __forceinline__ void rel_shared(const P64 &P, const double *f, int i, int j, double &f3, double &a1,
                                           double &a2, double &a3, double &cor) {
    const int pit = P.pitch;
    f3 = f[pidx(i, j, pit)];
    const double m0 = 0.104166666666667, m1 = -0.708333333333334, m2 = 0.708333333333334, m3 = -0.104166666666667;
    const double m4 = 0.117647058823529, m5 = 0.029411764705882, m6 = 0.029411764705882, m7 = 0.117647058823529;
    const double m8 = -0.083333333333333, m9 = 0.166666666666667, m10 = -0.166666666666667, m11 = 0.083333333333334;
    double g1 = f[pidx(i - 2, j, pit)] - f3;
    double g2 = f[pidx(i - 1, j, pit)] - f3;
    double g4 = f[pidx(i + 1, j, pit)] - f3;
    double g5 = f[pidx(i + 2, j, pit)] - f3;
    a1 = m0 * g1 + m1 * g2 + m2 * g4 + m3 * g5;
    a2 = m4 * g1 + m5 * g2 + m6 * g4 + m7 * g5;
    a3 = m8 * g1 + m9 * g2 + m10 * g4 + m11 * g5;
    double te = 0.0;
    for (int q = 0; q < P.rtb; q++) {
        double v = P.relc[3 * q] * a1 + P.relc[3 * q + 1] * a2 + P.relc[3 * q + 2] * a3 + f3;
        te += v;
    }
    cor = f3 - (1.0 / (double)P.rtb) * te;
}
__device__ __forceinline__ double rel_pick(const P64 &P, int k, double a1, double a2, double a3, double f3) {
    return P.relc[3 * k] * a1 + P.relc[3 * k + 1] * a2 + P.relc[3 * k + 2] * a3 + f3;
}
// The same two for the fast FP64 form: multiply-adds fused (this file is otherwise
// compiled without contraction).
__device__ __forceinline__ void rel_shared_fma(const P64 &P, const double *f, int i, int j, double &f3, double &a1,
                                               double &a2, double &a3, double &cor) {
    const int pit = P.pitch;
    f3 = f[pidx(i, j, pit)];
    const double m0 = 0.104166666666667, m1 = -0.708333333333334, m2 = 0.708333333333334, m3 = -0.104166666666667;
    const double m4 = 0.117647058823529, m5 = 0.029411764705882, m6 = 0.029411764705882, m7 = 0.117647058823529;
    const double m8 = -0.083333333333333, m9 = 0.166666666666667, m10 = -0.166666666666667, m11 = 0.083333333333334;
    const double g1 = f[pidx(i - 2, j, pit)] - f3, g2 = f[pidx(i - 1, j, pit)] - f3;
    const double g4 = f[pidx(i + 1, j, pit)] - f3, g5 = f[pidx(i + 2, j, pit)] - f3;
    a1 = __fma_rn(m3, g5, __fma_rn(m2, g4, __fma_rn(m1, g2, m0 * g1)));
    a2 = __fma_rn(m7, g5, __fma_rn(m6, g4, __fma_rn(m5, g2, m4 * g1)));
    a3 = __fma_rn(m11, g5, __fma_rn(m10, g4, __fma_rn(m9, g2, m8 * g1)));
    double te = 0.0;
    for (int q = 0; q < P.rtb; q++)
        te += __fma_rn(P.relc[3 * q + 2], a3, __fma_rn(P.relc[3 * q + 1], a2, __fma_rn(P.relc[3 * q], a1, f3)));
    cor = __fma_rn(-1.0 / (double)P.rtb, te, f3);
}
__device__ __forceinline__ double rel_pick_fma(const P64 &P, int k, double a1, double a2, double a3, double f3) {
    return __fma_rn(P.relc[3 * k + 2], a3, __fma_rn(P.relc[3 * k + 1], a2, __fma_rn(P.relc[3 * k], a1, f3)));
}

__device__ __forceinline__ double cell_asq(const RunFields &F, int x) {
    int i = x + F.pre;
    i = i > -1 ? i : 0;
    i = i < F.nf ? i : F.nf - 1;
    double ay = F.Ay[F.nf + i], az = F.Az[F.nf + i];
    return (ay * ay) + (az * az);
}

// One warp per coarse column i, kMomCols columns of one patch per block; a warp forms
// its column's finest sub-columns k in pairs, the f stencil and the interpolation's
// shared part once per cell for the pair.  The warp walks p in windows of 32 lanes
// covering j0-1 .. j0+30: every lane computes the Lorentz factor at its p-face once
// (shared with the neighbouring face through shuffles instead of the reference's four
// Gamma calls per cell), the log ratio
//   L(j) = c2 * ln((g_{j+1} + c1 p_{j+1}) / (g_j + c1 p_j))
// (the reference's gm; gm1 and gp1 are L(j-1) and L(j+1), the same expressions), the
// interpolated f and the cell's charge/current contributions.  The window's 29
// contributions per sub-column then go through shared memory to the block's last warp,
// whose lanes each add one sub-column's in ascending j, which keeps the reference's
// accumulation order (Rectangle.cpp:207-255) exactly.  The serial sums thus take one
// FP64 warp instruction per cell for up to 30 sub-columns at once (an FP64 warp
// instruction occupies the sub-partition's FP64 unit for tens of cycles whatever the
// number of active lanes), and with two window buffers they run while the column warps
// form the next window.
// The coarse-column list is padded per patch to a multiple of kMomCols (padding: patch
// -1), so the warps of a block share n_p and rtb and step through the windows together.
constexpr int kMomOut = kMomWindow;  // outputs per window: j0 .. j0+28
constexpr int kMomThreads = (kMomCols + 1) * 32;

// Two window buffers: the column warps fill one while the summing warp adds the other.
struct MomSmem {
    double cc[2][kMomCols][2][32], cj[2][kMomCols][2][32];
    unsigned use[2][kMomCols];
};

// Barrier of one moment unit's kMomThreads threads: barrier 0 in k64_moments (the whole
// block), named barriers 1 and 2 for the two units a pipelined block carries.
__device__ __forceinline__ void mom_sync(int bar) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(kMomThreads) : "memory");
}

// One window of column i's sub-columns k0 .. k0+kg-1 (kg <= 2): lane L covers the p index
// j = j0 - 1 + L; lanes 1 .. kMomOut return the charge and current contributions cc[q],
// cj[q] of their cell (zero where the cell is not used) and set `use`.  All 32 lanes
// take part (shuffles).  a[q]: q^2 A^2 of sub-column k0+q.
// ln(Gn / G) for the fast FP64 form.  Neighbouring nodes of a p grid differ by a factor
// 1 + dp / gamma, so z = (Gn - G) / (Gn + G) is small and ln(Gn / G) = 2 atanh(z) =
// 2 z (1 + z^2/3 + z^4/5 + z^6/7) to within z^8 / 9 < 1.2e-17 relative for |z| <= 0.01;
// otherwise (and for G = 0 past the window's end, whose value is not used) the logarithm
// of the quotient.
__device__ __forceinline__ double fast_log_ratio(double Gn, double G) {
    const double s = Gn + G;
    if (G != 0.0 && s != 0.0) {
        const double z = (Gn - G) * rcp_nr(s);
        if (fabs(z) <= 0.01) {
            const double z2 = z * z;
            const double poly = __fma_rn(z2, __fma_rn(z2, __fma_rn(z2, 1.0 / 7.0, 0.2), 1.0 / 3.0), 1.0);
            return (2.0 * z) * poly;
        }
        return log(Gn * rcp_nr(G));
    }
    return log(Gn / G);
}

// FAST (the fast FP64 form): multiply-adds fused and the node ratio's logarithm as above;
// the same formulas, not the reference's rounding.
template <bool FAST>
__device__ __forceinline__ void mom_window(const P64 &P, const double *f, bool real, int i, int j0, int k0, int kg,
                                           const double a[2], double c1, double c2, int lane, double cc[2],
                                           double cj[2], bool &use) {
    const unsigned full = 0xffffffffu;
    const double c3 = 1 / 48.0;
    const int np = P.np, rtb = P.rtb, pit = P.pitch;
    const int j = j0 - 1 + lane;  // this lane's p index
    double p = 0.0, f3 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0, cor = 0.0;
    use = false;
    if (real) {
        p = FAST ? __fma_rn(P.dp, (double)(j + P.p_pos), P.pmin) : P.pmin + P.dp * (double)(j + P.p_pos);
        if (j <= np) {
            if (rtb == 1) f3 = f[pidx(i, j, pit)];
            else if (FAST) rel_shared_fma(P, f, i, j, f3, a1, a2, a3, cor);
            else rel_shared(P, f, i, j, f3, a1, a2, a3, cor);
        }
        use = lane >= 1 && lane <= kMomOut && j < np && !(P.nested && P.nested[pidx(i, j, pit)]);
    }
    for (int q = 0; q < kg; q++) {
        cc[q] = 0.0;
        cj[q] = 0.0;
        if (real) {
            double G = 0.0, V = 0.0;
            if (j <= np + 1) {
                if (FAST) {
                    const double g = sqrt(__fma_rn(__fma_rn(p, p, a[q]), P.g2, 1.0));
                    G = __fma_rn(c1, p, g);
                } else {
                    double g = sqrt(1.0 + ((p * p) + a[q]) * P.g2);
                    G = g + c1 * p;
                }
            }
            if (j <= np) V = rtb == 1 ? f3 : (FAST ? rel_pick_fma(P, k0 + q, a1, a2, a3, f3) : rel_pick(P, k0 + q, a1, a2, a3, f3)) + cor;
            const double Gn = __shfl_down_sync(full, G, 1);
            // valid for lanes 0..30 (lane 31's Gn is its own G; beyond n_p + 1, G = 0)
            const double L = FAST ? c2 * fast_log_ratio(Gn, G) : c2 * log(Gn / G);
            const double Lm = __shfl_up_sync(full, L, 1);
            const double Lp = __shfl_down_sync(full, L, 1);
            const double Vm = __shfl_up_sync(full, V, 1);
            const double Vp = __shfl_down_sync(full, V, 1);
            if (use) {
                cc[q] = V;
                cj[q] = FAST ? __fma_rn(V, L, c3 * (Lp - Lm) * (Vp - Vm)) : V * L + c3 * (Lp - Lm) * (Vp - Vm);
            }
        }
    }
}

// One unit: the kMomCols columns col0 .. col0 + kMomCols - 1 of the padded column list,
// formed by warps 0 .. kMomCols - 1 and summed by warp kMomCols (wid: warp within the unit).
template <bool FAST>
__device__ __forceinline__ void moments_unit(const MomLaunch &M, int col0, int wid, int lane, MomSmem &S, int bar) {
    const bool summer = wid == kMomCols;  // the last warp adds; warps 0..kMomCols-1 form columns
    const bool real = !summer && M.colpatch[col0 + wid] >= 0;  // warp-uniform
    const P64 &P = ((const P64 *)M.patches)[M.colpatch[col0]];  // the unit's patch
    const int np = P.np, rtb = P.rtb;
    const int i = summer ? 0 : M.colidx[col0 + wid] / rtb;
    const RunFields &F = M.fields[P.run];
    const double minv = 1 / P.mass;
    const double c1 = minv * kCInv;
    const double c2 = 1 / c1;
    const double *f = P.f1;
    const unsigned full = 0xffffffffu;
    for (int k0 = 0; k0 < rtb; k0 += 2) {  // unit-uniform
        const int kg = rtb - k0 < 2 ? rtb - k0 : 2;
        double a[2] = {0.0, 0.0};
        for (int q = 0; q < kg; q++)
            if (real) a[q] = P.qq * cell_asq(F, (i + P.x_pos) * rtb + k0 + q);
        // summing warp, lane t < kMomCols * kg: sub-column t % kg of column t / kg
        double ch = 0.0, cu = 0.0;
        auto add_window = [&](int bf) {
            if (lane < kMomCols * kg) {
                const int w = lane / kg, q = lane - w * kg;
                const unsigned um = S.use[bf][w];
                for (int t = 1; t <= kMomOut; t++)
                    if ((um >> t) & 1u) {
                        ch += S.cc[bf][w][q][t];
                        cu += S.cj[bf][w][q][t];
                    }
            }
        };
        int bf = 0;
        for (int j0 = 0; j0 < np; j0 += kMomOut, bf ^= 1) {
            if (!summer) {
                double cc[2], cj[2];
                bool use;
                mom_window<FAST>(P, f, real, i, j0, k0, kg, a, c1, c2, lane, cc, cj, use);
                for (int q = 0; q < kg; q++) {
                    S.cc[bf][wid][q][lane] = cc[q];
                    S.cj[bf][wid][q][lane] = cj[q];
                }
                const unsigned usemask = __ballot_sync(full, use);
                if (lane == 0) S.use[bf][wid] = usemask;
            } else if (j0 > 0) {
                add_window(bf ^ 1);  // the previous window, in ascending j
            }
            mom_sync(bar);
        }
        if (summer) {
            add_window(bf ^ 1);  // the last window
            if (lane < kMomCols * kg) {
                const int w = lane / kg, q = lane - w * kg;
                if (M.colpatch[col0 + w] >= 0) {
                    const int cl = M.colidx[col0 + w] + k0 + q;  // i_w * rtb + k
                    const double qc = P.q;
                    P.chargeR[cl] = ch * (P.dp * qc);
                    P.currentR[cl] = cu * (-qc * qc / P.mass);
                }
            }
        }
        mom_sync(bar);  // the next pair's first window reuses the buffers
    }
}

template <bool FAST>
__global__ void __launch_bounds__(kMomThreads, 2) k64_moments(MomLaunch M) {
    VX_PDL_WAIT();
    __shared__ MomSmem S;
    moments_unit<FAST>(M, blockIdx.x * kMomCols, threadIdx.x >> 5, threadIdx.x & 31, S, 0);
}

void launch_moments64(const MomLaunch &M) {
    if (M.ncols == 0) return;
    // M.ncols is a multiple of kMomCols (the list is padded per patch)
    if (M.fast) vx_launch(k64_moments<true>, M.ncols / kMomCols, kMomThreads, 0, M.stream, M);
    else vx_launch(k64_moments<false>, M.ncols / kMomCols, kMomThreads, 0, M.stream, M);
}

// ---------------------------------------------------------------- separable initial f
// Interior cells of an FP32 patch's slots 0 and 1: (float)(((dx_sum[i] dp_sum[j]) inv) fn),
// the host quadrature's product in its order (this file keeps IEEE multiplies unfused).
__global__ void k_fill_separable(float *f0, float *f1, int pitch, int nx, int np, const double *dx_sum,
                                 const double *dp_sum, double inv, double fn) {
    VX_PDL_WAIT();
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= np || i >= nx) return;
    const double v = dx_sum[i] * dp_sum[j] * inv;
    const float x = (float)(v * fn);
    const int id = pidx(i, j, pitch);
    f0[id] = x;
    f1[id] = x;
}

void launch_fill_separable(float *f0, float *f1, int pitch, int nx, int np, const double *dx_sum,
                           const double *dp_sum, double inv, double fn, cudaStream_t s) {
    vx_launch(k_fill_separable, dim3((np + 255) / 256, nx), 256, 0, s, f0, f1, pitch, nx, np, dx_sum, dp_sum, inv, fn);
}

// Rectangle::InitializeDistribution (Rectangle.cpp:616-665) for a problem whose
// InitialDistribution is a sum of product terms, f(x, p) = sum_t (X_t(x) * P_t(p)) / C_t.
// The host evaluates the hook's factors at every sample point (X over the patch's n_x *
// nvals x samples, P over its n_p * nvals p samples, with its own exp / sin); each
// thread forms one cell's nvals^2 samples in the reference's loop order and operation
// order (--fmad=false: no contraction), so the cell averages equal the host loop's bits.
__global__ void k64_quadrature(double *f0, double *f1, int pitch, int nx, int np, int nvals, int terms,
                               const double *X, const double *Pf, const double *C, double scale) {
    VX_PDL_WAIT();
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= np || i >= nx) return;
    const double *xr = X + (size_t)i * nvals, *pr = Pf + (size_t)j * nvals;
    const size_t xstride = (size_t)nx * nvals, pstride = (size_t)np * nvals;
    double temp = 0.0;
    for (int k = 0; k < nvals; k++) {
        for (int l = 0; l < nvals; l++) {
            double v = (xr[k] * pr[l]) / C[0];
            for (int t = 1; t < terms; t++) v = v + (xr[t * xstride + k] * pr[t * pstride + l]) / C[t];
            temp = temp + v;
        }
    }
    const double f = temp * scale;
    const int id = pidx(i, j, pitch);
    f0[id] = f;
    f1[id] = f;
}

void launch_quadrature64(double *f0, double *f1, int pitch, int nx, int np, int nvals, int terms, const double *X,
                         const double *Pf, const double *C, double scale, cudaStream_t s) {
    vx_launch(k64_quadrature, dim3((np + 127) / 128, nx), 128, 0, s, f0, f1, pitch, nx, np, nvals, terms, X, Pf, C,
              scale);
}

// ---------------------------------------------------------------- assembly
// FP64 runs; runs of the FP32 form go to launch_assemble32 (stage32.cu).
__global__ void k_assemble(AsmLaunch A) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (run >= A.nruns) return;
    assemble_cell(A, run, x);
}

void launch_assemble(const AsmLaunch &A) {
    if (A.pairs) {
        launch_assemble32(A);
        return;
    }
    dim3 g((A.maxn + 255) / 256, A.nruns);
    vx_launch(k_assemble, g, 256, 0, A.stream, A);
}

// ---------------------------------------------------------------- Poisson
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
    return -fcoef * (8 * (phi[ip1] - phi[im1]) - phi[ip2] + phi[im2]) + ex0;
}

// One block per run.  The triangular solves are linear recurrences; to keep the
// reference's rounding they run in one thread in the order of the column-oriented
// dgetrs (entries ascending in column for L, descending for U).  FP64 dependent latency
// (~64 cycles per add/mul, ~550 per IEEE division on this part) makes the chain length
// the cost, so the factors are stored in band form: four coefficients per row for the
// columns next to the diagonal (exact zeros where the factor has none — subtracting a
// zero product never changes a partial sum, which is never -0 here) plus a short list of
// "far" entries that precede the band in the summation order.  Only the product with the
// previous row's value sits on the critical path.  Back substitution divides with
// Markstein's sequence (q = s*y, r = s - q*u exactly, q' = q + r*y with y = RN(1/u));
// after each chunk the whole block checks every quotient against the IEEE quotient and
// the chunk is redone with IEEE division if any differs, so the result is always the
// dgetrs rounding.
constexpr int kPoisRows = kPoisRowsHost;     // rows per chunk
constexpr int kPoisLA = 4;                   // look-ahead rows staged with each chunk
constexpr int kPoisBuf = kPoisRows + kPoisLA;
constexpr int kPoisFar = 2048;               // far entries per staged chunk

struct PoisBandChunk {
    int a;                                    // first staged row
    double c[4][kPoisBuf];                    // band coefficients, c[d-1][row - a]
    double diag[kPoisBuf], rdiag[kPoisBuf], rdlo[kPoisBuf];  // U only
    double num[kPoisRows], rhs[kPoisRows];    // backward: numerators, chunk right-hand sides
    double slotc[4][kPoisBuf];                // forward: accumulator-lane coefficients per step
    int sload[4][kPoisBuf];                   // forward: row taken up by each slot at each step
    int take[kPoisBuf];                       // forward: slot finishing row step+4
    int fptr[kPoisBuf + 1];
    int fcol[kPoisFar];
    double fval[kPoisFar];
};

// Stage rows [a, b) (clamped to [0, n)) of a band factor into B with threads
// [t0, t0+nt).  Returns whether the far entries fit.
__device__ bool pois_stage_band(PoisBandChunk &B, const BandFactor &F, int a, int b, int n, int t0, int nt,
                                bool upper) {
    a = max(a, 0);
    b = min(b, n);
    const int cnt = b - a;
    const int f0 = F.fptr[a], f1 = F.fptr[b];
    const bool fits = (f1 - f0) <= kPoisFar;
    const int t = (int)threadIdx.x - t0;
    if (t == 0) B.a = a;
    for (int k = t; k < cnt; k += nt) {
        const int r = a + k;
        B.c[0][k] = F.band[4 * r];
        B.c[1][k] = F.band[4 * r + 1];
        B.c[2][k] = F.band[4 * r + 2];
        B.c[3][k] = F.band[4 * r + 3];
        if (upper) {
            B.diag[k] = F.diag[r];
            B.rdiag[k] = F.rdiag[r];
            B.rdlo[k] = F.rdiag_lo[r];
        }
        for (int sl = 0; sl < F.nslots; sl++) {
            B.slotc[sl][k] = F.slot_coef[(size_t)sl * n + r];
            B.sload[sl][k] = F.slot_load[(size_t)sl * n + r];
        }
        if (F.take) B.take[k] = F.take[r];
    }
    // buffer rows past n: neutral entries, so that a look-ahead read past the matrix's end
    // finds a zero coefficient and no row index
    for (int k = cnt + t; k < kPoisBuf; k += nt) {
        B.c[0][k] = B.c[1][k] = B.c[2][k] = B.c[3][k] = 0.0;
        for (int sl = 0; sl < 4; sl++) {  // every accumulator row of the buffer
            B.slotc[sl][k] = 0.0;
            B.sload[sl][k] = -1;
        }
        B.take[k] = -1;
    }
    for (int k = t; k <= cnt; k += nt) B.fptr[k] = F.fptr[a + k] - f0;
    if (fits)
        for (int e = f0 + t; e < f1; e += nt) {
            B.fcol[e - f0] = F.fcol[e];
            B.fval[e - f0] = F.fval[e];
        }
    return fits;
}

// Right-hand side of row r with its far entries subtracted in summation order.
template <bool FAR_SMEM>
__device__ __forceinline__ double pois_far(const PoisBandChunk &B, const BandFactor &F, const double *x, int r) {
    const int k = r - B.a;
    double s = x[r];
    const int gbase = FAR_SMEM ? 0 : F.fptr[B.a];
    for (int e = B.fptr[k]; e < B.fptr[k + 1]; e++) {
        const int col = FAR_SMEM ? B.fcol[e] : F.fcol[gbase + e];
        const double v = FAR_SMEM ? B.fval[e] : F.fval[gbase + e];
        s = s - x[col] * v;
    }
    return s;
}

// Software-pipelined substitution on lanes 0..3 of warp 0.  Row i's sum is
// ((((Fb - x4 c4) - x3 c3) - x2 c2) - x1 c1), x_d the solution d rows back (forward) or
// ahead (backward), Fb the right-hand side minus its far entries.  Lane L holds the
// partial sum of row i+L (forward) / i-L (backward), already reduced by every term but
// the one with x_{i-1} (x_{i+1}); when that value arrives, each lane subtracts its own
// product in the same two warp instructions, lane 0's result is x_i (before the division
// backward), and the partials shift down one lane while lane 3 takes up the next row's
// right-hand side.  On this part each FP64 warp instruction occupies the sub-partition's
// FP64 unit for tens of cycles whatever the number of active lanes, so the lanes carry
// the independent work for free.
template <bool FAR_SMEM>
__device__ void pois_fwd_chunk(const PoisBandChunk &B, const BandFactor &F, int r0, int cnt, int n, double *x,
                               double &V, double &w1) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int L = lane < 4 ? lane : 3;
    const int slot = lane - 4;  // lanes 4..7: accumulators of the rows with far terms
    const bool is_slot = slot >= 0 && slot < F.nslots;
    const bool slots = F.nslots >= 0;
    // Operands of row r0 + q, loaded one row ahead so their shared-memory latency overlaps
    // the previous row's multiply-subtract.
    auto fetch = [&](int q, double &coef, int &ld, double &fb, int &tk) {
        const int i = r0 + q;
        const int k = i - B.a;
        coef = 0.0;
        ld = -1;
        if (lane < 4) coef = (i + L < n) ? B.c[L][k + L] : 0.0;
        else if (is_slot) {
            ld = B.sload[slot][k];
            coef = B.slotc[slot][k];
        }
        fb = 0.0;
        if (slots && lane == 3 && i + 4 < n) fb = x[i + 4];
        tk = slots ? B.take[k] : -1;
    };
    double coef, fb;
    int ld, tk;
    fetch(0, coef, ld, fb, tk);
    for (int q = 0; q < cnt; q++) {
        const int i = r0 + q;
        if (ld >= 0) V = x[ld];  // a slot takes up a new row's right-hand side
        if (!slots && lane == 3 && i + 4 < n) fb = pois_far<FAR_SMEM>(B, F, x, i + 4);
        const double nv = V - w1 * coef;
        double coef_n = 0.0, fb_n = 0.0;
        int ld_n = -1, tk_n = -1;
        if (q + 1 < cnt) fetch(q + 1, coef_n, ld_n, fb_n, tk_n);
        const double xi = __shfl_sync(full, nv, 0);
        const double up = __shfl_down_sync(full, nv, 1);
        if (slots) {
            const double fin = __shfl_sync(full, nv, 4 + (tk >= 0 ? tk : 0));
            if (tk >= 0) fb = fin;
        }
        V = (lane == 3) ? fb : (is_slot ? nv : up);
        if (lane == 0) x[i] = xi;
        if (!slots) __syncwarp();  // lane 3 reads x[i] when it gathers a later row's far entries
        w1 = xi;
        coef = coef_n;
        fb = fb_n;
        ld = ld_n;
        tk = tk_n;
    }
}

template <bool FAR_SMEM, bool IEEE>
__device__ void pois_bwd_chunk(PoisBandChunk &B, const BandFactor &F, int r0, int cnt, double *x, double &V,
                               double &w1, bool far_done) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int L = lane < 4 ? lane : 3;
    auto fetch = [&](int qq, double &coef, double &fb, double &u, double &y) {
        const int i = r0 + qq;
        const int k = i - B.a;
        coef = (i - L >= 0) ? B.c[L][k - L] : 0.0;
        fb = (far_done && lane == 3 && i - 4 >= 0) ? x[i - 4] : 0.0;
        u = B.diag[k];
        y = B.rdiag[k];
    };
    double coef, fb, u, y;
    fetch(cnt - 1, coef, fb, u, y);
    for (int qq = cnt - 1; qq >= 0; qq--) {
        const int i = r0 + qq;
        if (!far_done && lane == 3 && i - 4 >= 0) fb = pois_far<FAR_SMEM>(B, F, x, i - 4);
        const double nv = V - w1 * coef;
        double coef_n = 0.0, fb_n = 0.0, u_n = 1.0, y_n = 1.0;
        if (qq > 0) fetch(qq - 1, coef_n, fb_n, u_n, y_n);
        const double up = __shfl_down_sync(full, nv, 1);
        double xi = 0.0;
        if (lane == 0) {
            if (IEEE) {
                xi = nv / u;
            } else {
                B.num[qq] = nv;
                xi = __fma_rn(nv, y, __dmul_rn(nv, B.rdlo[i - B.a]));
            }
            x[i] = xi;
        }
        xi = __shfl_sync(full, xi, 0);
        if (!far_done) __syncwarp();  // lane 3 reads x[i] when it gathers a later row's far entries
        V = (lane == 3) ? fb : up;
        w1 = xi;
        coef = coef_n;
        fb = fb_n;
        u = u_n;
        y = y_n;
    }
}

// Steady-state forms of the two chunk loops (every far term handled by accumulator
// lanes or by the parallel pass): each lane walks its own coefficient stream with a
// pointer, the shift and the slot hand-over are one shuffle with a per-lane source, and
// no branch depends on the lane.  The operands of the next row are loaded at the top of
// each row, ahead of its multiply: the warp issues in order, and a load placed after the
// previous row's shuffle-dependent store would add its shared-memory latency to every row
// of the chain (forward 282 -> 242 cycles per row, step 28.4 -> 27.1 ms).  The look-ahead
// reads at most two rows past the chunk: the staged look-ahead rows, or past n the
// neutral entries pois_stage_band writes there (zero coefficients, no slot row).
__device__ void pois_fwd_fast(const PoisBandChunk &B, const BandFactor &F, int r0, int cnt, int n, double *x,
                              double &V, double &w1) {
    // Only lanes 0..7 (band lanes 0..3, accumulator lanes 4..7) run the recurrence.
    constexpr unsigned act = 0xffu;
    const int lane = threadIdx.x & 31;
    if (lane >= 8) return;
    const int slot = lane - 4;
    const bool is_slot = slot >= 0 && slot < F.nslots;
    const bool has_coef = lane < 4 || is_slot;
    const int k0 = r0 - B.a;
    // coefficient stream of this lane (lanes without a role read slot 0's and use zero)
    const double *cp = lane < 4 ? &B.c[lane][k0 + lane] : &B.slotc[is_slot ? slot : 0][k0];
    const int cstep = has_coef ? 1 : 0;
    // row indices the slot takes up, read two rows ahead so that x[row] is one row ahead
    const int *lp = &B.sload[is_slot ? slot : 0][k0];
    const int lstep = is_slot ? 1 : 0;
    const int base_src = lane < 3 ? lane + 1 : lane;
    // rows past the end of the matrix get a zero coefficient
    const int lim = lane < 4 ? n - 1 - lane - r0 : cnt;  // q > lim: row i+lane >= n
    double coef = (0 > lim || !has_coef) ? 0.0 : *cp;
    cp += cstep;
    int ld = is_slot ? *lp : -1;
    lp += lstep;
    int ldn = is_slot ? *lp : -1;
    lp += lstep;
    double vld = ld >= 0 ? x[ld] : 0.0;
    int tk = B.take[k0];
    double fb = (lane == 3 && r0 + 4 < n) ? x[r0 + 4] : 0.0;
    for (int q = 0; q < cnt; q++) {
        const int i = r0 + q;
        // row q+1's operands; a slot's row r >= step + 4 and the right-hand side x[i + 5]
        // are not yet overwritten by the sweep.  Rows past the chunk read the staged
        // look-ahead rows, or past n the neutral entries pois_stage_band leaves there.
        double coef_n = *cp;
        cp += cstep;
        if (q + 1 > lim || !has_coef) coef_n = 0.0;
        const int tk_n = B.take[k0 + q + 1];
        const double fb_n = (lane == 3 && i + 5 < n) ? x[i + 5] : 0.0;
        const double vld_n = ldn >= 0 ? x[ldn] : 0.0;
        const int ldnn = is_slot ? *lp : -1;
        lp += lstep;
        if (ld >= 0) V = vld;  // a slot takes up a new row's right-hand side
        const double nv = V - w1 * coef;
        const double xi = __shfl_sync(act, nv, 0, 8);
        const int src = (lane == 3 && tk >= 0) ? 4 + tk : base_src;  // tk < kMaxSlots = 4
        const double sh = __shfl_sync(act, nv, src, 8);
        V = (lane == 3 && tk < 0) ? fb : sh;
        if (lane == 0) x[i] = xi;
        w1 = xi;
        coef = coef_n;
        tk = tk_n;
        fb = fb_n;
        vld = vld_n;
        ld = ldn;
        ldn = ldnn;
    }
}

__device__ void pois_bwd_fast(PoisBandChunk &B, int r0, int cnt, double *x, double &V, double &w1) {
    // Lanes 0..3 run the multiply-subtract and lane 0 alone the quotient (the same
    // instructions on four lanes made the backward sweep 40 % slower); the other lanes
    // leave V and w1 unused.
    constexpr unsigned act = 0xfu;
    const int lane = threadIdx.x & 31;
    if (lane >= 4) return;
    const int L = lane;
    const int kl = r0 + cnt - 1 - B.a;  // buffer row of the chunk's last (first processed) row
    const double *cp = &B.c[L][kl - L];
    const double *yp = &B.rdiag[kl];
    const double *lp = &B.rdlo[kl];
    const int ilast = r0 + cnt - 1;
    double coef = (ilast - L < 0) ? 0.0 : cp[0];
    double y = yp[0], ylo = lp[0];
    cp--;
    yp--;
    lp--;
    double fb = (lane == 3 && ilast - 4 >= 0) ? x[ilast - 4] : 0.0;
    for (int qq = cnt - 1; qq >= 0; qq--) {
        const int i = r0 + qq;
        // row i-1's operands (kPoisLA rows are staged below the chunk); x[i - 5] is still
        // the right-hand side
        const double coef_n = (i - 1 - L >= 0) ? cp[0] : 0.0;
        const double y_n = qq > 0 ? yp[0] : 0.0, ylo_n = qq > 0 ? lp[0] : 0.0;
        const double fb_n = (lane == 3 && i - 5 >= 0) ? x[i - 5] : 0.0;
        cp--;
        yp--;
        lp--;
        const double nv = V - w1 * coef;
        const double up = __shfl_down_sync(act, nv, 1, 4);
        // quotient from the reciprocal split into high and low parts: within 2^-105 of
        // nv/u before the final rounding; the chunk check catches the rare wrong rounding
        double q1 = 0.0;
        if (lane == 0) {
            q1 = __fma_rn(nv, y, __dmul_rn(nv, ylo));
            B.num[qq] = nv;
            x[i] = q1;
        }
        const double xi = __shfl_sync(act, q1, 0, 4);
        V = (lane == 3) ? fb : up;
        w1 = xi;
        coef = coef_n;
        y = y_n;
        ylo = ylo_n;
        fb = fb_n;
    }
}

constexpr int kPoisSmemMaxN = 16384;  // solution vector kept in shared memory up to this n

// ---- pipelined form: the solve follows the moment units of its run (k64_moments_poisson)
constexpr unsigned kPipeMaxPolls = 1u << 25;  // second bound of a wait (>= 64 ns per poll)

__device__ __forceinline__ unsigned long long pipe_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned pipe_ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int pipe_ld_relaxed(const int *p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void pipe_bar(int bar, int nt) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nt) : "memory");
}

// Waits until done counter ci has every unit it expects.  A wait that runs out records
// itself in *err and returns; so does every later wait at once (the step's values are
// then not valid, but every index stays what the host tables say: nothing goes out of
// bounds).
__device__ void pipe_wait(const PipeLaunch &K, int ci) {
    const unsigned need = (unsigned)K.need[ci] + (unsigned)K.phantom;
    const unsigned *p = K.state + kPipeDone + ci;
    if (pipe_ld_acquire(p) >= need) return;
    if (pipe_ld_relaxed(K.err) != 0) return;
    const unsigned long long t0 = pipe_ns();
    for (unsigned poll = 0;; poll++) {
        __nanosleep(32);
        if (pipe_ld_acquire(p) >= need) break;
        if ((poll & 63u) == 63u && pipe_ld_relaxed(K.err) != 0) break;
        if (poll >= kPipeMaxPolls || pipe_ns() - t0 > K.limit_ns) {
            atomicCAS(K.err, 0, 1 + ci);
            break;
        }
    }
    __threadfence();
}

// Rows that forward chunk c reads first: one thread waits for the chunk's moment units,
// then threads t = 0 .. nt-1 (barrier bar) assemble rho and J at each row's x position
// perm[k] and form its right-hand side as the unpipelined solve does
// (tmp[i] = (te * (charge[i] + neut[i])) * w, then x[k] = tmp[perm[k]]).  off_sp0: while
// warp 0 runs the sweep, the FP64 work stays off its sub-partition (warps 4m), whose FP64
// unit the sweep's dependent chain needs.
__device__ void pipe_rows(const PipeLaunch &K, int run, int c, double *x, int t, int nt, int bar, bool off_sp0) {
    if (t == 0) {
        if (K.trace && run == 0 && c == 0) K.trace[0] = pipe_ns();
        pipe_wait(K, K.run_ctr[run] + c);
        if (K.trace && run == 0) K.trace[1 + c] = pipe_ns();
    }
    pipe_bar(bar, nt);
    const int *gp = K.gptr + K.run_gptr[run];
    RunFields &F = K.P.fields[run];
    const int *perm = K.P.lu[run].perm;
    const double te = kEps0Inv;
    const double w = K.P.w[run];
    if (off_sp0) {  // warps 1..31 of the block: the 24 that are not 4m
        const int wg = (int)threadIdx.x >> 5;
        if ((wg & 3) == 0) return;
        t = ((wg >> 2) * 3 + (wg & 3) - 1) * 32 + ((int)threadIdx.x & 31);
        nt = 24 * 32;
    }
    for (int e = gp[c] + t; e < gp[c + 1]; e += nt) {
        const int k = K.grow[e], i = perm[k];
        assemble_cell<true>(K.A, run, i);
        const double v = te * (F.charge[i] + F.neut[i]);
        x[k] = v * w;
    }
}

// The solve with the solution vector x in shared memory (XS) or in phi itself.  The two
// instantiations let the compiler see x's address space: with one pointer chosen at run
// time its loads and stores in the sweeps go through generic addressing.
template <bool XS, bool PIPE>
__device__ __forceinline__ void poisson_solve(const PoissonLaunch &L, unsigned char *smem_raw, double *x,
                                              const PipeLaunch *K) {
    PoisBandChunk *buf = (PoisBandChunk *)smem_raw;  // two chunk buffers, then the solution vector
    __shared__ int s_bad;
    const int run = blockIdx.x;
    RunFields &F = L.fields[run];
    const LUDev &lu = L.lu[run];
    const int n = F.n;
    constexpr bool in_smem = XS;
    double *tmp = F.efin;  // scratch until E_x is recomputed at the end
    const double te = kEps0Inv;
    const double w = L.w[run];
    if (PIPE) {
        pipe_rows(*K, run, 0, x, threadIdx.x, blockDim.x, 0, false);  // chunk 0's rows, all threads
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double v = te * (F.charge[i] + F.neut[i]);
            tmp[i] = v * w;
        }
        __syncthreads();
        // Row interchanges of dgetrs applied as one gather: b'[k] = b[perm[k]].
        for (int k = threadIdx.x; k < n; k += blockDim.x) x[k] = tmp[lu.perm[k]];
    }
    const int nchunks = (n + kPoisRows - 1) / kPoisRows;
    unsigned long long *trace = (L.trace && run == 0 && threadIdx.x == 0) ? L.trace : nullptr;
    // clock64 (cycles) alone; globaltimer (ns) when pipelined, to compare with the moment units
    auto tick = [] { return PIPE ? pipe_ns() : (unsigned long long)clock64(); };
    if (trace) trace[0] = tick();
    if (PIPE && K->trace && run == 0 && threadIdx.x == 0) K->trace[1 + 2 * K->trace_nch] = clock64();
    const int lane = threadIdx.x & 31;
    // ---- forward: rows ascending; chunk c stages rows [c*R, c*R + R + LA)
    {
        double V = 0.0, w1 = 0.0;
        bool fit_cur = pois_stage_band(buf[0], lu.L, 0, kPoisBuf, n, 0, blockDim.x, false);
        __syncthreads();
        if (threadIdx.x < 32 && lane < 4 && lane < n)
            V = fit_cur ? pois_far<true>(buf[0], lu.L, x, lane) : pois_far<false>(buf[0], lu.L, x, lane);

        if (PIPE) {
            // warp 0 sweeps, the others stage the next chunk and gather its rows: two
            // loops with one block barrier per chunk each, so that the sweep's loop holds
            // only the sweep's values (the accumulator-lane form: the host pipelines only
            // factors that have it)
            if (threadIdx.x < 32) {
                for (int c = 0; c < nchunks; c++) {
                    const int r0 = c * kPoisRows;
                    pois_fwd_fast(buf[c & 1], lu.L, r0, min(kPoisRows, n - r0), n, x, V, w1);
                    __syncthreads();
                    if (trace) trace[1 + c] = tick();
                }
            } else {
                for (int c = 0; c + 1 < nchunks; c++) {
                    const int r1 = (c + 1) * kPoisRows;
                    pois_stage_band(buf[(c + 1) & 1], lu.L, r1, r1 + kPoisBuf, n, 32, blockDim.x - 32, false);
                    // the rows chunk c+1 reads first, while warp 0 sweeps chunk c (it reads
                    // and writes only rows first read by chunks up to c)
                    pipe_rows(*K, run, c + 1, x, threadIdx.x - 32, blockDim.x - 32, 1, true);
                    __syncthreads();
                }
                __syncthreads();  // the last chunk's
            }
        }
        for (int c = 0; !PIPE && c < nchunks; c++) {
            const int r0 = c * kPoisRows, cnt = min(kPoisRows, n - r0);
            PoisBandChunk &B = buf[c & 1];
            bool fit_next = false;
            if (c + 1 < nchunks) {
                const int r1 = r0 + kPoisRows;
                if (threadIdx.x >= 32)
                    fit_next = pois_stage_band(buf[(c + 1) & 1], lu.L, r1, r1 + kPoisBuf, n, 32, blockDim.x - 32, false);
                else
                    fit_next = (lu.L.fptr[min(r1 + kPoisBuf, n)] - lu.L.fptr[r1]) <= kPoisFar;
            }
            if (threadIdx.x < 32) {
                if (lu.L.nslots >= 0) pois_fwd_fast(B, lu.L, r0, cnt, n, x, V, w1);
                else if (fit_cur) pois_fwd_chunk<true>(B, lu.L, r0, cnt, n, x, V, w1);
                else pois_fwd_chunk<false>(B, lu.L, r0, cnt, n, x, V, w1);
            }
            fit_cur = fit_next;
            __syncthreads();
            if (trace) trace[1 + c] = tick();
        }
    }
    if (PIPE && K->trace && run == 0 && threadIdx.x == 0) K->trace[2 + 2 * K->trace_nch] = clock64();
    // ---- backward: rows descending; chunk c stages rows [c*R - LA, c*R + R)
    {
        double V = 0.0, w1 = 0.0;
        bool far_done = false;
        const int clast = nchunks - 1;
        int parity = 0;
        bool fit_cur = pois_stage_band(buf[0], lu.U, clast * kPoisRows - kPoisLA, n, n, 0, blockDim.x, true);
        __syncthreads();
        if (threadIdx.x < 32 && lane < 4 && n - 1 - lane >= 0)
            V = fit_cur ? pois_far<true>(buf[0], lu.U, x, n - 1 - lane) : pois_far<false>(buf[0], lu.U, x, n - 1 - lane);
        for (int c = clast; c >= 0; c--) {
            const int r0 = c * kPoisRows, cnt = min(kPoisRows, n - r0);
            PoisBandChunk &B = buf[parity];
            bool fit_next = false;
            if (c > 0) {
                const int r1 = (c - 1) * kPoisRows;
                if (threadIdx.x >= 32)
                    fit_next = pois_stage_band(buf[parity ^ 1], lu.U, r1 - kPoisLA, r1 + kPoisRows, n, 32, blockDim.x - 32, true);
                else
                    fit_next = (lu.U.fptr[r1 + kPoisRows] - lu.U.fptr[max(r1 - kPoisLA, 0)]) <= kPoisFar;
            }
            const double V0 = V, w10 = w1;
            if (threadIdx.x < 32) {
                if (threadIdx.x == 0) s_bad = 0;
                for (int q = lane; q < cnt; q += 32) B.rhs[q] = x[r0 + q];
                __syncwarp();
                if (far_done) pois_bwd_fast(B, r0, cnt, x, V, w1);
                else if (fit_cur) pois_bwd_chunk<true, false>(B, lu.U, r0, cnt, x, V, w1, far_done);
                else pois_bwd_chunk<false, false>(B, lu.U, r0, cnt, x, V, w1, far_done);
            }
            __syncthreads();
            // every Markstein quotient of the chunk against the IEEE quotient of its numerator
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
                const double ieee = B.num[q] / B.diag[r0 + q - B.a];
                if (__double_as_longlong(ieee) != __double_as_longlong(x[r0 + q])) s_bad = 1;
            }
            __syncthreads();
            if (s_bad && threadIdx.x < 32) {
                for (int q = lane; q < cnt; q += 32) x[r0 + q] = B.rhs[q];
                __syncwarp();
                V = V0;
                w1 = w10;
                if (fit_cur) pois_bwd_chunk<true, true>(B, lu.U, r0, cnt, x, V, w1, far_done);
                else pois_bwd_chunk<false, true>(B, lu.U, r0, cnt, x, V, w1, far_done);
            }
            __syncthreads();
            if (!far_done && c == clast && lu.U.far_pre_col == r0 && r0 > 4) {
                // x_{r0..n-1} are final: subtract the far terms of every row below r0-4 at once
                for (int r = threadIdx.x; r < r0 - 4; r += blockDim.x) {
                    double v = x[r];
                    for (int e = lu.U.fptr[r]; e < lu.U.fptr[r + 1]; e++) v = v - x[lu.U.fcol[e]] * lu.U.fval[e];
                    x[r] = v;
                }
                far_done = true;
            }
            fit_cur = fit_next;
            parity ^= 1;
            __syncthreads();
            if (trace) trace[1 + nchunks + (clast - c)] = tick();
        }
    }
    if (in_smem)
        for (int i = threadIdx.x; i < n; i += blockDim.x) F.phi[i] = x[i];
    if (threadIdx.x == 0) {
        double ex0 = *F.ex0;
        double e_m1 = efield_at(x, n, L.fcoef[run], ex0, -1);
        double e_0 = efield_at(x, n, L.fcoef[run], ex0, 0);
        *F.ex0 = ex0 + -(e_m1 + e_0) * 0.5;
    }
    __syncthreads();
    const double ex0 = *F.ex0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) F.efin[i] = efield_at(x, n, L.fcoef[run], ex0, i);
}

__global__ void __launch_bounds__(1024, 1) k_poisson(PoissonLaunch L) {
    VX_PDL_WAIT();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (L.x_in_smem) poisson_solve<true, false>(L, smem_raw, (double *)(smem_raw + 2 * sizeof(PoisBandChunk)), nullptr);
    else poisson_solve<false, false>(L, smem_raw, L.fields[blockIdx.x].phi, nullptr);
}

// ---- workers of the pipelined launch
// One item: column warp wid forms window j0 of its column's sub-columns k0, k0+1 (those
// the patch has) and writes the contributions of lanes 1 .. kMomOut to `out`.
template <bool FAST>
__device__ __forceinline__ void mom_item(const PipeLaunch &K, int u, int k0, int j0, int wid, int lane, double *out) {
    const MomLaunch &M = K.M;
    const int col0 = K.unit_col0[u];
    const bool real = M.colpatch[col0 + wid] >= 0;  // warp-uniform
    const P64 &P = ((const P64 *)M.patches)[M.colpatch[col0]];
    const int rtb = P.rtb;
    const int i = M.colidx[col0 + wid] / rtb;
    const RunFields &F = M.fields[P.run];
    const double2 c12 = K.unit_c12[u];
    const int kg = rtb - k0 < 2 ? rtb - k0 : 2;
    double a[2] = {0.0, 0.0};
    for (int q = 0; q < kg; q++)
        if (real) a[q] = P.qq * cell_asq(F, (i + P.x_pos) * rtb + k0 + q);
    double cc[2], cj[2];
    bool use;
    mom_window<FAST>(P, P.f1, real, i, j0, k0, kg, a, c12.x, c12.y, lane, cc, cj, use);
    if (lane >= 1 && lane <= kMomOut)
        for (int q = 0; q < kg; q++) {
            out[lane * 30 + wid * 2 + q] = cc[q];
            out[960 + lane * 30 + wid * 2 + q] = cj[q];
        }
}

// The column sums of unit u (one warp, lane = sub-column as in k64_moments): every window's
// contributions in ascending p.  A cell that is not used contributes +0.0, which leaves a
// sum that starts at +0.0 unchanged bit for bit (such a sum never becomes -0.0), so these
// are the sums of the used cells alone.  Then the unit counts as done for its chunk.
__device__ void mom_sum_unit(const PipeLaunch &K, int u, int lane) {
    const MomLaunch &M = K.M;
    const int col0 = K.unit_col0[u];
    const P64 &P = ((const P64 *)M.patches)[M.colpatch[col0]];
    const int rtb = P.rtb, nw = K.unit_nwin[u];
    for (int k0 = 0; k0 < rtb; k0 += 2) {
        const int kg = rtb - k0 < 2 ? rtb - k0 : 2;
        if (lane < kMomCols * kg) {
            const int w = lane / kg, q = lane - w * kg;
            const double *src = K.scratch + (size_t)(K.unit_item0[u] + (k0 / 2) * nw) * kPipeItemDoubles + w * 2 + q;
            double ch = 0.0, cu = 0.0;
            for (int win = 0; win < nw; win++, src += kPipeItemDoubles) {
#pragma unroll
                for (int t = 1; t <= kMomOut; t++) {
                    ch += __ldcg(src + t * 30);
                    cu += __ldcg(src + 960 + t * 30);
                }
            }
            if (M.colpatch[col0 + w] >= 0) {
                const int cl = M.colidx[col0 + w] + k0 + q;  // i_w * rtb + k
                const double qc = P.q;
                P.chargeR[cl] = ch * (P.dp * qc);
                P.currentR[cl] = cu * (-qc * qc / P.mass);
            }
        }
    }
    __threadfence();  // the column sums, device-wide, before the count
    __syncwarp();
    if (lane == 0) {
        atomicAdd(K.state + kPipeDone + K.unit_sig[u], 1u);
        if (K.trace && K.unit_sig[u] < K.trace_nch) atomicMax(K.trace + 1 + K.trace_nch + K.unit_sig[u], pipe_ns());
    }
}

// A group of a worker block: column warps 0 .. kMomCols-1 take items until none are left;
// the warp that completes a unit (the unit's item count reaches its total) appends the
// unit to the queue of completed units.  They never wait for anything but each other.
template <bool FAST>
__device__ void pipe_columns(const PipeLaunch &K, int *ticket, int g) {
    const int tid = (int)threadIdx.x - g * kMomThreads, wid = tid >> 5, lane = tid & 31;
    const int bar = 1 + g, ncol = kMomCols * 32;
    unsigned *items_done = K.state + kPipeDone + K.ndone;      // per unit
    unsigned *queue = items_done + K.nunits;                    // completed units (u + 1), in order
    for (int it = 0;; it++) {
        if (tid == 0) ticket[it & 1] = (int)atomicAdd(K.state + kPipeTicket, 1u);
        pipe_bar(bar, ncol);
        const int t = ticket[it & 1];
        if (t >= K.nitems) break;
        const int u = K.item_unit[t];
        const int loc = t - K.unit_item0[u], nw = K.unit_nwin[u];
        const int kp = loc / nw;
        mom_item<FAST>(K, u, 2 * kp, (loc - kp * nw) * kMomOut, wid, lane, K.scratch + (size_t)t * kPipeItemDoubles);
        __threadfence();  // this warp's contributions, device-wide, before the item counts
        pipe_bar(bar, ncol);
        if (tid == 0) {
            const unsigned total = (unsigned)(K.unit_item0[u + 1] - K.unit_item0[u]);
            if (atomicAdd(items_done + u, 1u) + 1 == total) {
                __threadfence();  // every item's contributions before a summing warp reads them
                const unsigned slot = atomicAdd(K.state + kPipeQHead, 1u);
                atomicExch(queue + slot, (unsigned)u + 1);
            }
        }
    }
}

// A summing warp (one per sub-partition of a summing block, so that its serial adds have
// the sub-partition's FP64 unit to themselves): takes completed units from the queue in
// order and forms their column sums.  It waits only for units, which the column warps
// always complete; a wait that runs out records itself and ends the warp.
__device__ void pipe_summer(const PipeLaunch &K, int lane) {
    const unsigned full = 0xffffffffu;
    unsigned *queue = K.state + kPipeDone + K.ndone + K.nunits;
    for (;;) {
        int slot = 0;
        if (lane == 0) slot = (int)atomicAdd(K.state + kPipeQTail, 1u);
        slot = __shfl_sync(full, slot, 0);
        if (slot >= K.nunits) break;
        unsigned v = 0;
        if (lane == 0) {
            v = pipe_ld_acquire(queue + slot);
            if (!v) {
                const unsigned long long t0 = pipe_ns();
                for (unsigned poll = 0;; poll++) {
                    __nanosleep(64);
                    v = pipe_ld_acquire(queue + slot);
                    if (v) break;
                    if ((poll & 63u) == 63u && pipe_ld_relaxed(K.err) != 0) break;
                    if (poll >= kPipeMaxPolls || pipe_ns() - t0 > K.limit_ns) {
                        atomicCAS(K.err, 0, 1 + K.ndone);
                        break;
                    }
                }
            }
        }
        v = __shfl_sync(full, v, 0);
        if (!v) break;
        __threadfence();
        mom_sum_unit(K, (int)v - 1, lane);
    }
}

// Moments, assembly and the exact solve in one launch.  Block r < nruns solves run r (its
// forward sweep starts as soon as the moments of its first rows are summed, instead of
// after the whole moments kernel); the next K.summers blocks carry four summing warps each
// (pipe_summer); every other block carries two groups of column warps (pipe_columns).
// Column warps wait for nothing outside their group, summing warps only for column
// warps, the solve only for summing warps: every wait ends whatever order the blocks are
// scheduled in.  Same arithmetic as k64_moments + k_assemble + k_poisson.
template <bool FAST>
__global__ void __launch_bounds__(1024, 1) k64_moments_poisson(PipeLaunch K) {
    VX_PDL_WAIT();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if ((int)blockIdx.x < K.P.nruns) {
        if (K.P.x_in_smem)
            poisson_solve<true, true>(K.P, smem_raw, (double *)(smem_raw + 2 * sizeof(PoisBandChunk)), &K);
        else poisson_solve<false, true>(K.P, smem_raw, K.P.fields[blockIdx.x].phi, &K);
    } else if ((int)blockIdx.x < K.P.nruns + K.summers) {
        if (threadIdx.x < 4 * 32) pipe_summer(K, (int)threadIdx.x & 31);  // warps 0..3: one per sub-partition
    } else {
        int *ticket = reinterpret_cast<int *>(smem_raw);
        const int g = (int)threadIdx.x / kMomThreads;
        if (((int)threadIdx.x & (kMomThreads - 1)) < kMomCols * 32) pipe_columns<FAST>(K, ticket + 2 * g, g);
    }
    // the last block out zeroes the tickets, the queue, done and item counters for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(K.state + kPipeLeave, 1u) + 1 == gridDim.x) {
            atomicExch(K.state + kPipeTicket, 0u);
            atomicExch(K.state + kPipeQHead, 0u);
            atomicExch(K.state + kPipeQTail, 0u);
            for (int i = 0; i < K.ndone + 2 * K.nunits; i++) atomicExch(K.state + kPipeDone + i, 0u);
            atomicExch(K.state + kPipeLeave, 0u);
            __threadfence();
        }
    }
}

void launch_poisson(const PoissonLaunch &L) {
    PoissonLaunch P = L;
    int max_smem = 0, dev = 0;  // per call: engines on several host threads may launch
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    // the solution vector joins the two chunk buffers in shared memory when it fits
    const int base = 2 * (int)sizeof(PoisBandChunk);
    P.x_in_smem = (L.maxn <= kPoisSmemMaxN && base + 8 * L.maxn <= max_smem) ? 1 : 0;
    const int smem = base + (P.x_in_smem ? 8 * L.maxn : 0);
    cudaFuncSetAttribute(k_poisson, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // 1024 threads x 64 registers take a whole SM's register file: no block of the FP64
    // face kernels that run beside the solve shares the SM, whose FP64 unit would
    // otherwise delay the solve's dependent chain (step 32.4 -> 28.1 ms on 4096 x 512)
    vx_launch(k_poisson, L.nruns, 1024, smem, L.stream, P);
}

void launch_moments_poisson64(const PipeLaunch &K0) {
    PipeLaunch K = K0;
    int max_smem = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int base = 2 * (int)sizeof(PoisBandChunk);
    K.P.x_in_smem = (K.P.maxn <= kPoisSmemMaxN && base + 8 * K.P.maxn <= max_smem) ? 1 : 0;
    const int smem_solve = base + (K.P.x_in_smem ? 8 * K.P.maxn : 0);
    const int smem = std::max(smem_solve, 16);
    auto kern = K.M.fast ? k64_moments_poisson<true> : k64_moments_poisson<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(K.P.nruns + K.summers + K.workers);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = K.stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributePriority;
    attr[0].val.priority = K.priority;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = g_launch_pdl ? 2 : 1;
    cudaLaunchKernelEx(&cfg, kern, K);  // errors surface through cudaGetLastError
}

// E_x on the finest grid from phi and Ex0 (EMSolver::GetEfield), for states loaded from
// outside the step.
__global__ void k_efield(RunFields *fields, const double *fcoef, int nruns, int f32) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= nruns) return;
    RunFields &F = fields[run];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n) return;
    const double e = efield_at(F.phi, F.n, fcoef[run], *F.ex0, i);
    F.efin[i] = e;
    if (f32) F.efin32[i] = (float)e;
}

void launch_efield(RunFields *fields, const double *fcoef, int nruns, int maxn, int f32, cudaStream_t s) {
    dim3 g((maxn + 255) / 256, nruns);
    vx_launch(k_efield, g, 256, 0, s, fields, fcoef, nruns, f32);
}

// ---------------------------------------------------------------- Maxwell
// FP64 runs; runs of the FP32 form go to launch_maxwell32 (stage32.cu).
__global__ void k_mx_rhs(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_rhs_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_mx_update(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_update_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void k_mx_asq(MaxwellLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    if (run >= L.nruns) return;
    mx_asq_cell(L, run, blockIdx.x * blockDim.x + threadIdx.x);
}

void launch_maxwell(const MaxwellLaunch &L) {
    if (L.f32) {
        launch_maxwell32(L);
        return;
    }
    dim3 g((L.maxnf + 255) / 256, L.nruns);
    vx_launch(k_mx_rhs, g, 256, 0, L.stream, L);
    vx_launch(k_mx_update, g, 256, 0, L.stream, L);
    vx_launch(k_mx_asq, g, 256, 0, L.stream, L);
}

// ---------------------------------------------------------------- CFL
// The maximum runs over non-negative doubles, so it is taken on their bit patterns:
// each block reduces its slice and folds it into out[run] with an integer atomicMax.
__global__ void k_cfl(CflLaunch L) {
    VX_PDL_WAIT();
    const int run = blockIdx.y;
    const RunFields &F = L.fields[run];
    const int ns = L.run_ns[run];
    const double *sp = L.spec + run * 25;  // up to 8 species x 3 + dpsMax
    const double dpsMax = sp[24];
    __shared__ double red[256];
    double pc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F.n; i += gridDim.x * blockDim.x) {
        double Azv = F.Az[i], Ayv = F.Ay[i];
        double As = Ayv * Ayv + Azv * Azv;
        double temp = 0.0;
        for (int j = 0; j < ns; j++) {
            double aq = sp[3 * j], m = sp[3 * j + 1], dps = sp[3 * j + 2];
            double v = aq / m / sqrt(1 + As / ((m * kCs) * (m * kCs))) * dps;
            temp = (temp < v) ? v : temp;
        }
        double v = temp * fabs(Ayv * F.Bz[i] - Azv * F.By[i]) + dpsMax * fabs(F.efin[i]);
        pc = (pc < v) ? v : pc;
    }
    red[threadIdx.x] = pc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            double o = red[threadIdx.x + s];
            red[threadIdx.x] = (red[threadIdx.x] < o) ? o : red[threadIdx.x];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        atomicMax((unsigned long long *)&L.out[run], (unsigned long long)__double_as_longlong(red[0]));
}

void launch_cfl(const CflLaunch &L) {
    cudaMemsetAsync(L.out, 0, (size_t)L.nruns * sizeof(double), L.stream);
    dim3 g(std::min(32, std::max(1, (L.maxn + 255) / 256)), L.nruns);
    vx_launch(k_cfl, g, 256, 0, L.stream, L);
}

__global__ void k_negate(double *dst, const double *src, int n) {
    VX_PDL_WAIT();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = -src[i];
}

void launch_negate(double *dst, const double *src, int n, cudaStream_t s) {
    vx_launch(k_negate, (n + 255) / 256, 256, 0, s, dst, src, n);
}

}  // namespace vx

namespace vx {
// Eight independent fused multiply-add chains per thread (register resident).  The
// result is stored so the chains are not eliminated.
__global__ void k_fp64_peak(double *out, int iters) {
    VX_PDL_WAIT();
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
    double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
    const double b = 0.999999, c = 1e-7;
    for (int k = 0; k < iters; k++) {
        a0 = fma(a0, b, c);
        a1 = fma(a1, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
        a5 = fma(a5, b, c);
        a6 = fma(a6, b, c);
        a7 = fma(a7, b, c);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

void launch_fp64_peak(double *out, int blocks, int threads, int iters, cudaStream_t s) {
    vx_launch(k_fp64_peak, blocks, threads, 0, s, out, iters);
}

// Dependent-chain latency on one lane: iters steps of the substitution's multiply-
// subtract, then the same with a 64-bit shuffle in the chain (clock64 cycles, into
// cyc[0] and cyc[1]; the chains' values into val so that they are not eliminated).
__global__ void k_fp64_latency(long long *cyc, double *val, int iters) {
    VX_PDL_WAIT();
    double x = 1.0 + threadIdx.x * 1e-3;
    const double c = 0.999999, v = 1e-7;
    long long t0 = clock64();
    for (int k = 0; k < iters; k++) x = v - x * c;
    long long t1 = clock64();
    double y = x;
    for (int k = 0; k < iters; k++) {
        y = v - y * c;
        y = __shfl_sync(0xffffffffu, y, 0);
    }
    long long t2 = clock64();
    if (threadIdx.x == 0) {
        cyc[0] = t1 - t0;
        cyc[1] = t2 - t1;
        val[0] = x + y;
    }
}

void launch_fp64_latency(long long *cyc, double *val, int iters, cudaStream_t s) {
    vx_launch(k_fp64_latency, 1, 32, 0, s, cyc, val, iters);
}
}  // namespace vx
