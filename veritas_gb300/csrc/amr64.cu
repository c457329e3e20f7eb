// Device execution of the AMR op lists built in amr.cpp.  Each launch runs one batch of
// ops that touch disjoint cells; the batches run in order on the context stream.
// Compiled with --fmad=false: every expression keeps the reference's operation order.
#include <cuda_runtime.h>

#include "amr.hpp"
#include "vx_kernels.hpp"

namespace vx {

using P64 = PatchT<double>;

__device__ __forceinline__ double *slot_plane(const P64 &P, int slot) {
    return slot == 0 ? P.f0 : (slot == 1 ? P.f1 : P.f2);
}

__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }  // std::min

// Rectangle::GetInterpolantsREF (Rectangle.cpp:121-137): r values from five cells.
__device__ __forceinline__ void interp_ref(const double *c, int r, double f1, double f2, double f3, double f4, double f5,
                                          double *out) {
    const double m0 = 0.104166666666667, m1 = -0.708333333333334, m2 = 0.708333333333334, m3 = -0.104166666666667;
    const double m4 = 0.117647058823529, m5 = 0.029411764705882, m6 = 0.029411764705882, m7 = 0.117647058823529;
    const double m8 = -0.083333333333333, m9 = 0.166666666666667, m10 = -0.166666666666667, m11 = 0.083333333333334;
    f5 -= f3;
    f4 -= f3;
    f2 -= f3;
    f1 -= f3;
    double a1 = m0 * f1 + m1 * f2 + m2 * f4 + m3 * f5;
    double a2 = m4 * f1 + m5 * f2 + m6 * f4 + m7 * f5;
    double a3 = m8 * f1 + m9 * f2 + m10 * f4 + m11 * f5;
    for (int i = 0; i < r; i++) out[i] = c[3 * i] * a1 + c[3 * i + 1] * a2 + c[3 * i + 2] * a3 + f3;
}

constexpr int kMaxR = 8;

// Rectangle::GetWenoValueFromCoarseLevel (Rectangle.cpp:343-415): entry `sub` of the
// corrected r x r interpolants of coarse cell (ic, jc).
__device__ double coarse_interp(const P64 &C, const double *f, int ic, int jc, int sub) {
    const int r = C.r;
    const int pit = C.pitch;
    double temps[5][kMaxR];
    for (int k = -2; k < 3; k++)
        interp_ref(C.refc, r, f[pidx(ic - 2, jc + k, pit)], f[pidx(ic - 1, jc + k, pit)], f[pidx(ic, jc + k, pit)],
                   f[pidx(ic + 1, jc + k, pit)], f[pidx(ic + 2, jc + k, pit)], temps[k + 2]);
    double sum = 0.0, want = 0.0;
    for (int k = 0; k < r; k++) {
        double part[kMaxR];
        interp_ref(C.refc, r, temps[0][k], temps[1][k], temps[2][k], temps[3][k], temps[4][k], part);
        for (int l = 0; l < r; l++) {
            sum += part[l];
            if (k * r + l == sub) want = part[l];
        }
    }
    double correction = f[pidx(ic, jc, pit)] - 1.0 / pow((double)r, 2.0) * sum;
    return want + correction;
}

__global__ void k_ghost(const P64 *patches, const GhostOp *ops, int n, int slot) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const GhostOp op = ops[k];
    const P64 &D = patches[op.dst];
    double v = 0.0;
    if (op.kind == kGhostCopy) {
        const P64 &S = patches[op.src];
        v = slot_plane(S, slot)[pidx(op.si, op.sj, S.pitch)];
    } else if (op.kind == kGhostRestrict) {  // Rectangle::GetValueFromFinerLevel (Rectangle.cpp:314-327)
        const P64 &S = patches[op.src];
        const double *f = slot_plane(S, slot);
        const int r = D.r;
        double t = 0.0;
        for (int a = 0; a < r; a++)
            for (int b = 0; b < r; b++) t += f[pidx(op.si + a, op.sj + b, S.pitch)];
        t /= pow((double)r, 2.0);
        v = t;
    } else if (op.kind == kGhostInterp) {
        const P64 &S = patches[op.src];
        v = coarse_interp(S, slot_plane(S, slot), op.si, op.sj, op.sub);
    }
    slot_plane(D, slot)[pidx(op.di, op.dj, D.pitch)] = v;
}

// Coarse faces on a coarse/fine interface: the mean of the finer patch's fluxes through
// the r fine faces (CalculateFluxToCoarse*, Rectangle.hpp:132-178).  The high-order mean
// uses the fine patch's stage fluxes; the stage-0 low-order mean recomputes each fine
// donor-cell flux the way RGKGetFluxXL/PL do, (dx_inv * f) * a (Rectangle.cpp:1216-1253).
__global__ void k_iface(const P64 *patches, const IfaceOp *ops, int n, int step) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const IfaceOp op = ops[k];
    const P64 &C = patches[op.coarse];
    const P64 &F = patches[op.fine];
    const int r = C.r;
    const int cid = pidx(op.ci, op.cj, C.pitch);
    const double scale = 1.0 / (r * r);
    const double *f = F.f1;
    if (op.dir == 0) {
        double t = 0.0;
        for (int q = 0; q < r; q++) t += F.FxH[step][pidx(op.fi, op.fj + q, F.pitch)];
        C.FxH[step][cid] = t * scale;
        if (step == 0) {
            double tl = 0.0;
            for (int q = 0; q < r; q++) {
                const int fid = pidx(op.fi, op.fj + q, F.pitch);
                double lo;
                if (F.ifx && F.ifx[fid]) lo = F.FxL[fid];
                else {
                    const double am = F.ex[fid];
                    lo = F.dx_inv * (am > 0.0 ? f[fid - F.pitch] : f[fid]) * am;
                }
                tl += lo;
            }
            C.FxL[cid] = tl * scale;
        }
    } else {
        double t = 0.0;
        for (int q = 0; q < r; q++) t += F.FpH[step][pidx(op.fi + q, op.fj, F.pitch)];
        C.FpH[step][cid] = t * scale;
        if (step == 0) {
            double tl = 0.0;
            for (int q = 0; q < r; q++) {
                const int fid = pidx(op.fi + q, op.fj, F.pitch);
                double lo;
                if (F.ifp && F.ifp[fid]) lo = F.FpL[fid];
                else {
                    const double am = F.ep[fid];
                    lo = F.dp_inv * (am > 0.0 ? f[fid - 1] : f[fid]) * am;
                }
                tl += lo;
            }
            C.FpL[cid] = tl * scale;
        }
    }
}

// Limiter coefficient exchange (Rectangle.cpp:1625-1917).
__global__ void k_csync(const P64 *patches, const CSyncOp *ops, int n) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const CSyncOp op = ops[k];
    const P64 &N = patches[op.nb];
    const P64 &R = patches[op.caller];
    const int t = op.t;
    const bool xf = t < 2;
    double *NC = xf ? N.Cx : N.Cp;
    double *RC = xf ? R.Cx : R.Cp;
    const double *NDS = xf ? N.FxDS : N.FpDS;
    const double *RDS = xf ? R.FxDS : R.FpDS;
    const int nid = pidx(op.ni, op.nj, N.pitch);
    const int cid = pidx(op.ci, op.cj, R.pitch);
    const int nprev = xf ? nid - N.pitch : nid - 1;  // (ni-1, nj) or (ni, nj-1)
    const int cprev = xf ? cid - R.pitch : cid - 1;
    if (op.kind == kCSame) {  // SetCFromSameLevel
        double v;
        if (t == 0 || t == 2)
            v = NDS[nid] > 0.0 ? dmin(R.Rp[cid], N.Rm[nprev]) : dmin(N.Rp[nprev], R.Rm[cid]);
        else
            v = NDS[nid] > 0.0 ? dmin(R.Rm[cprev], N.Rp[nid]) : dmin(N.Rm[nid], R.Rp[cprev]);
        NC[nid] = v;
        RC[cid] = v;
    } else if (op.kind == kCUpdate) {  // UpdateCFromSameLevel
        double v = dmin(NC[nid], RC[cid]);
        NC[nid] = v;
        RC[cid] = v;
    } else {  // SetCFromDifferentLevel
        const int r = N.r;
        double v = NC[nid];
        for (int q = 0; q < r; q++) {
            const int fid = xf ? cid + q : cid + q * R.pitch;
            const int fprev = xf ? fid - R.pitch : fid - 1;
            if (t == 0 || t == 2) v = dmin(v, RDS[fid] > 0.0 ? R.Rp[fid] : R.Rm[fid]);
            else v = dmin(v, RDS[fid] > 0.0 ? R.Rm[fprev] : R.Rp[fprev]);
        }
        if (t == 0 || t == 2) v = dmin(v, NDS[nid] > 0.0 ? N.Rm[nprev] : N.Rp[nprev]);
        else v = dmin(v, NDS[nid] > 0.0 ? N.Rp[nid] : N.Rm[nid]);
        for (int q = 0; q < r; q++) RC[xf ? cid + q : cid + q * R.pitch] = v;
        NC[nid] = v;
    }
}

void launch_ghost(const void *patches, const GhostOp *ops, int n, int slot, cudaStream_t s) {
    if (n <= 0) return;
    k_ghost<<<(n + 127) / 128, 128, 0, s>>>((const P64 *)patches, ops, n, slot);
}

void launch_iface(const void *patches, const IfaceOp *ops, int n, int step, cudaStream_t s) {
    if (n <= 0) return;
    k_iface<<<(n + 127) / 128, 128, 0, s>>>((const P64 *)patches, ops, n, step);
}

void launch_csync(const void *patches, const CSyncOp *ops, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_csync<<<(n + 127) / 128, 128, 0, s>>>((const P64 *)patches, ops, n);
}

}  // namespace vx
