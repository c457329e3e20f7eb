// Device bodies of the field-side stage work (one cell per call): the assembly of rho and
// J and the Maxwell RK stage.  Shared by fields64.cu (FP64 runs, compiled without
// contraction, so every expression keeps the reference's operation order) and stage32.cu
// (runs of the FP32 precision form, whose fields are FP64 too, compiled with contraction).
#pragma once
#include <cuda_runtime.h>

#include "vx_kernels.hpp"

namespace vx {

// ---------------------------------------------------------------- assembly
// Level::CollectRhoAndJ + EMFieldSolver::AssembleRhoAndJ (Level.cpp:19-62,
// EMSolver.cpp:104-122): per level, chargeL[x] = 0 + (patch values in patch order);
// charges_s[x] = 0 + level sums finest->coarsest; J sums species then levels;
// charge[x] = 0 + species sums.  CG: the column sums are read through L2 only (the
// pipelined solve reads them while the moment blocks that write them still run; see
// k64_moments_poisson).
template <bool CG = false>
__device__ __forceinline__ void assemble_cell(const AsmLaunch &A, int run, int x) {
    const int n = A.run_n[run];
    if (x >= n) return;
    const int ns = A.run_ns[run], nl = A.run_nl[run];
    const int *lp = A.lvl_ptr + A.lvl_off[run];
    const PatchT<double> *patches = (const PatchT<double> *)A.patches;
    double J = 0.0, charge = 0.0;
    for (int s = 0; s < ns; s++) {
        double cs = 0.0;
        for (int l = 0; l < nl; l++) {
            double lc = 0.0, lj = 0.0;
            for (int e = lp[s * nl + l]; e < lp[s * nl + l + 1]; e++) {
                const PatchT<double> &P = patches[A.lvl_patch[e]];
                int c = x - P.x_pos * P.rtb;
                if (c >= 0 && c < P.nx * P.rtb) {
                    if (A.pairs) {  // FP32 moments: (hi, lo) of the column sum, then its scale
                        const float2 qc = reinterpret_cast<const float2 *>(P.chargeR)[c];
                        const float2 qj = reinterpret_cast<const float2 *>(P.currentR)[c];
                        lc += ((double)qc.x + (double)qc.y) * P.msc_rho;
                        lj += ((double)qj.x + (double)qj.y) * P.msc_j;
                    } else if (CG) {
                        lc += __ldcg(P.chargeR + c);
                        lj += __ldcg(P.currentR + c);
                    } else {
                        lc += P.chargeR[c];
                        lj += P.currentR[c];
                    }
                }
            }
            cs += lc;
            J += lj;
        }
        charge += cs;
    }
    RunFields &F = A.fields[run];
    F.charge[x] = charge;
    F.J[x] = J;
}

// ---------------------------------------------------------------- Maxwell
// Right-hand side into slot step+2 from slot 1 (EMSolver.cpp:479-553).
__device__ __forceinline__ void mx_rhs_cell(const MaxwellLaunch &L, int run, int i) {
    RunFields &F = L.fields[run];
    const int nf = F.nf;
    if (i >= nf) return;
    const int s2 = (L.step + 2) * nf;
    const double *By = F.By + nf, *Bz = F.Bz + nf, *Ey = F.Ey + nf, *Ez = F.Ez + nf, *Ay = F.Ay + nf, *Az = F.Az + nf;
    const double dx_inv = L.dxinv[run];
    const double eps0_inv = kEps0Inv, mu_inv = kMuInv;
    double rBy = 0, rBz = 0, rEy = 0, rEz = 0, rAy = 0, rAz = 0;
    const int pre = F.pre, n = F.n;
    if (i == 0) {
        const double *pb = L.params + param_base(run, L.step);
        double by0 = pb[16], bz0 = pb[17];
        rBy = dx_inv * (Ez[1] - Ez[0]);
        rBz = -dx_inv * (Ey[1] - Ey[0]);
        rEy = -dx_inv * (Bz[0] - bz0) * eps0_inv * mu_inv;
        rEz = dx_inv * (By[0] - by0) * eps0_inv * mu_inv;
        rAy = -Ey[0];
        rAz = -Ez[0];
    } else if (i < pre || (i >= pre + n && i < nf - 2)) {
        rBy = dx_inv * (Ez[i + 1] - Ez[i]);
        rBz = -dx_inv * (Ey[i + 1] - Ey[i]);
        rEy = -dx_inv * (Bz[i] - Bz[i - 1]) * eps0_inv * mu_inv;
        rEz = dx_inv * (By[i] - By[i - 1]) * eps0_inv * mu_inv;
        rAy = -Ey[i];
        rAz = -Ez[i];
    } else if (i >= pre && i < pre + n) {
        const double c1 = -1.0 / 24;
        const double c2 = 9.0 / 8.0;
        const double Jv = F.J[i - pre];
        rBy = dx_inv * (c1 * (Ez[i + 2] - Ez[i - 1]) + c2 * (Ez[i + 1] - Ez[i]));
        rBz = -dx_inv * (c1 * (Ey[i + 2] - Ey[i - 1]) + c2 * (Ey[i + 1] - Ey[i]));
        rEy = -dx_inv * (c1 * (Bz[i + 1] - Bz[i - 2]) + c2 * (Bz[i] - Bz[i - 1])) * eps0_inv * mu_inv - eps0_inv * Jv * Ay[i];
        rEz = dx_inv * (c1 * (By[i + 1] - By[i - 2]) + c2 * (By[i] - By[i - 1])) * eps0_inv * mu_inv - eps0_inv * Jv * Az[i];
        rAy = -Ey[i];
        rAz = -Ez[i];
    }
    F.By[s2 + i] = rBy;
    F.Bz[s2 + i] = rBz;
    F.Ey[s2 + i] = rEy;
    F.Ez[s2 + i] = rEz;
    F.Ay[s2 + i] = rAy;
    F.Az[s2 + i] = rAz;
}

// Stage combination (EMSolver.cpp:204-338).  coef[0..5] are the dt-scaled weights of
// slots 2..7; the last stage writes slot 0 from slot 1 and copies it back to slot 1.
__device__ __forceinline__ void mx_combine(double *X, int nf, int i, int step, const double *c) {
    if (step < 5) {
        double v = X[i] + c[0] * X[2 * nf + i];
        for (int k = 1; k <= step; k++) v = v + c[k] * X[(k + 2) * nf + i];
        X[nf + i] = v;
    } else {
        double v = X[nf + i] + c[0] * X[2 * nf + i];
        for (int k = 1; k <= 5; k++) v = v + c[k] * X[(k + 2) * nf + i];
        X[i] = v;
        X[nf + i] = v;
    }
}

__device__ __forceinline__ void mx_update_cell(const MaxwellLaunch &L, int run, int i) {
    RunFields &F = L.fields[run];
    if (i >= F.nf) return;
    const double *c = L.params + param_base(run, L.step) + 8;
    mx_combine(F.By, F.nf, i, L.step, c);
    mx_combine(F.Bz, F.nf, i, L.step, c);
    mx_combine(F.Ey, F.nf, i, L.step, c);
    mx_combine(F.Ez, F.nf, i, L.step, c);
    mx_combine(F.Ay, F.nf, i, L.step, c);
    mx_combine(F.Az, F.nf, i, L.step, c);
    if (L.f32) {  // the per-cell A^2 the next stage's FP32 moments read (as acell32_cell), unfused
        const double ay = F.Ay[F.nf + i], az = F.Az[F.nf + i];
        F.acell32[i] = (float)__dadd_rn(__dmul_rn(ay, ay), __dmul_rn(az, az));
    }
}

// WENO-weighted (unmapped) face value of A (EMSolver.cpp:555-619).
__device__ __forceinline__ double face_a(double f1, double f2, double f3, double f4) {
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
    double oL = 0.5 / ((mm + bL) * (mm + bL));
    double oR = 0.5 / ((mm + bR) * (mm + bR));
    double wL = oL / (oL + oR);
    double wR = oR / (oL + oR);
    return wL * fL + wR * fR;
}

__device__ __forceinline__ void mx_asq_cell(const MaxwellLaunch &L, int run, int i) {
    RunFields &F = L.fields[run];
    if (i >= F.n) return;
    const double *Ay = F.Ay + F.nf + F.pre + i, *Az = F.Az + F.nf + F.pre + i;
    double a_y = face_a(Ay[-2], Ay[-1], Ay[0], Ay[1]);
    double a_z = face_a(Az[-2], Az[-1], Az[0], Az[1]);
    const double a = (a_y * a_y) + (a_z * a_z);
    F.asq[i] = a;
    if (L.asq32_out) F.asq32[i] = (float)a;
}

}  // namespace vx
