// Device execution of the AMR op lists built in amr.cpp.  Each launch runs one batch of
// ops that touch disjoint cells; the batches run in order on the context stream.
// Compiled with --fmad=false: every expression keeps the reference's operation order.
// Every kernel is instantiated for FP64 patches (the plain path) and FP32 patches (the
// precision form, arithmetic in FP32).
#include <cuda_runtime.h>

#include "amr.hpp"
#include "vx_kernels.hpp"

namespace vx {

template <class T>
__device__ __forceinline__ T *slot_plane(const PatchT<T> &P, int slot) {
    return slot == 0 ? P.f0 : (slot == 1 ? P.f1 : P.f2);
}

template <class T>
__device__ __forceinline__ T dmin(T a, T b) { return (b < a) ? b : a; }  // std::min

// Rectangle::GetInterpolantsREF (Rectangle.cpp:121-137): r values from five cells.
template <class T>
__device__ __forceinline__ void interp_ref(const double *c, int r, T f1, T f2, T f3, T f4, T f5, T *out) {
    const T m0 = (T)0.104166666666667, m1 = (T)-0.708333333333334, m2 = (T)0.708333333333334,
            m3 = (T)-0.104166666666667;
    const T m4 = (T)0.117647058823529, m5 = (T)0.029411764705882, m6 = (T)0.029411764705882,
            m7 = (T)0.117647058823529;
    const T m8 = (T)-0.083333333333333, m9 = (T)0.166666666666667, m10 = (T)-0.166666666666667,
            m11 = (T)0.083333333333334;
    f5 -= f3;
    f4 -= f3;
    f2 -= f3;
    f1 -= f3;
    T a1 = m0 * f1 + m1 * f2 + m2 * f4 + m3 * f5;
    T a2 = m4 * f1 + m5 * f2 + m6 * f4 + m7 * f5;
    T a3 = m8 * f1 + m9 * f2 + m10 * f4 + m11 * f5;
    for (int i = 0; i < r; i++) out[i] = (T)c[3 * i] * a1 + (T)c[3 * i + 1] * a2 + (T)c[3 * i + 2] * a3 + f3;
}

constexpr int kMaxR = 8;

// Rectangle::GetWenoValueFromCoarseLevel (Rectangle.cpp:343-415): the corrected r x r
// interpolants of coarse cell (ic, jc), out[kx * r + kp] for x sub-cell kx, p sub-cell kp.
template <class T>
__device__ void interp_block(const PatchT<T> &C, const T *f, int ic, int jc, T *out) {
    const int r = C.r;
    const int pit = C.pitch;
    T temps[5][kMaxR];
    for (int k = -2; k < 3; k++)
        interp_ref(C.refc, r, f[pidx(ic - 2, jc + k, pit)], f[pidx(ic - 1, jc + k, pit)], f[pidx(ic, jc + k, pit)],
                   f[pidx(ic + 1, jc + k, pit)], f[pidx(ic + 2, jc + k, pit)], temps[k + 2]);
    T sum = 0;
    for (int k = 0; k < r; k++) {
        interp_ref(C.refc, r, temps[0][k], temps[1][k], temps[2][k], temps[3][k], temps[4][k], out + k * r);
        for (int l = 0; l < r; l++) sum += out[k * r + l];
    }
    // 1 / r^2: r^2 is an exact small integer (the reference's std::pow(r, 2) gives it)
    T correction = f[pidx(ic, jc, pit)] - (T)1 / (T)(r * r) * sum;
    for (int q = 0; q < r * r; q++) out[q] += correction;
}

// Entry `sub` of interp_block.
template <class T>
__device__ T coarse_interp(const PatchT<T> &C, const T *f, int ic, int jc, int sub) {
    T out[kMaxR * kMaxR];
    interp_block(C, f, ic, jc, out);
    return out[sub];
}

template <class T>
__global__ void k_ghost(const PatchT<T> *patches, const GhostOp *ops, int n, int slot) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const GhostOp op = ops[k];
    const PatchT<T> &D = patches[op.dst];
    T v = 0;
    if (op.kind == kGhostCopy) {
        const PatchT<T> &S = patches[op.src];
        v = slot_plane(S, slot)[pidx(op.si, op.sj, S.pitch)];
    } else if (op.kind == kGhostRestrict) {  // Rectangle::GetValueFromFinerLevel (Rectangle.cpp:314-327)
        const PatchT<T> &S = patches[op.src];
        const T *f = slot_plane(S, slot);
        const int r = D.r;
        T t = 0;
        for (int a = 0; a < r; a++)
            for (int b = 0; b < r; b++) t += f[pidx(op.si + a, op.sj + b, S.pitch)];
        // std::pow(r, 2.0) of the reference, an exact integer; for a power of two the
        // product with its exact reciprocal is the same correctly rounded value
        if ((r & (r - 1)) == 0) t *= (T)(1.0 / (double)(r * r));
        else t /= (T)(r * r);
        v = t;
    } else if (op.kind == kGhostInterp) {
        const PatchT<T> &S = patches[op.src];
        v = coarse_interp(S, slot_plane(S, slot), op.si, op.sj, op.sub);
    }
    slot_plane(D, slot)[pidx(op.di, op.dj, D.pitch)] = v;
}

// Coarse faces on a coarse/fine interface: the mean of the finer patch's fluxes through
// the r fine faces (CalculateFluxToCoarse*, Rectangle.hpp:132-178).  The high-order mean
// uses the fine patch's stage fluxes; the stage-0 low-order mean recomputes each fine
// donor-cell flux the way RGKGetFluxXL/PL do, (dx_inv * f) * a (Rectangle.cpp:1216-1253).
template <class T>
__global__ void k_iface(const PatchT<T> *patches, const IfaceOp *ops, int n, int step) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const IfaceOp op = ops[k];
    const PatchT<T> &C = patches[op.coarse];
    const PatchT<T> &F = patches[op.fine];
    const int r = C.r;
    const int cid = pidx(op.ci, op.cj, C.pitch);
    const T scale = (T)(1.0 / (r * r));
    const T *f = F.f1;
    const T dxi = (T)F.dx_inv, dpi = (T)F.dp_inv;
    if (op.dir == 0) {
        T t = 0;
        for (int q = 0; q < r; q++) t += F.FxH[step][pidx(op.fi, op.fj + q, F.pitch)];
        C.FxH[step][cid] = t * scale;
        if (step == 0) {
            T tl = 0;
            for (int q = 0; q < r; q++) {
                const int fid = pidx(op.fi, op.fj + q, F.pitch);
                T lo;
                // the FP32 form keeps no face-velocity plane; its FxL is this value
                if (sizeof(T) == 4 || (F.ifx && F.ifx[fid])) lo = F.FxL[fid];
                else {
                    const T am = F.ex[fid];
                    lo = dxi * (am > (T)0 ? f[fid - F.pitch] : f[fid]) * am;
                }
                tl += lo;
            }
            C.FxL[cid] = tl * scale;
        }
    } else {
        T t = 0;
        for (int q = 0; q < r; q++) t += F.FpH[step][pidx(op.fi + q, op.fj, F.pitch)];
        C.FpH[step][cid] = t * scale;
        if (step == 0) {
            T tl = 0;
            for (int q = 0; q < r; q++) {
                const int fid = pidx(op.fi + q, op.fj, F.pitch);
                T lo;
                if (sizeof(T) == 4 || (F.ifp && F.ifp[fid])) lo = F.FpL[fid];
                else {
                    const T am = F.ep[fid];
                    lo = dpi * (am > (T)0 ? f[fid - 1] : f[fid]) * am;
                }
                tl += lo;
            }
            C.FpL[cid] = tl * scale;
        }
    }
}

// Limiter coefficient exchange (Rectangle.cpp:1625-1917).
template <class T>
__global__ void k_csync(const PatchT<T> *patches, const CSyncOp *ops, int n) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const CSyncOp op = ops[k];
    const PatchT<T> &N = patches[op.nb];
    const PatchT<T> &R = patches[op.caller];
    const int t = op.t;
    const bool xf = t < 2;
    T *NC = xf ? N.Cx : N.Cp;
    T *RC = xf ? R.Cx : R.Cp;
    const T *NDS = xf ? N.FxDS : N.FpDS;
    const T *RDS = xf ? R.FxDS : R.FpDS;
    const int nid = pidx(op.ni, op.nj, N.pitch);
    const int cid = pidx(op.ci, op.cj, R.pitch);
    const int nprev = xf ? nid - N.pitch : nid - 1;  // (ni-1, nj) or (ni, nj-1)
    const int cprev = xf ? cid - R.pitch : cid - 1;
    const T zero = 0;
    if (op.kind == kCSame) {  // SetCFromSameLevel
        T v;
        if (t == 0 || t == 2)
            v = NDS[nid] > zero ? dmin(R.Rp[cid], N.Rm[nprev]) : dmin(N.Rp[nprev], R.Rm[cid]);
        else
            v = NDS[nid] > zero ? dmin(R.Rm[cprev], N.Rp[nid]) : dmin(N.Rm[nid], R.Rp[cprev]);
        NC[nid] = v;
        RC[cid] = v;
    } else if (op.kind == kCUpdate) {  // UpdateCFromSameLevel
        T v = dmin(NC[nid], RC[cid]);
        NC[nid] = v;
        RC[cid] = v;
    } else {  // SetCFromDifferentLevel
        const int r = N.r;
        T v = NC[nid];
        for (int q = 0; q < r; q++) {
            const int fid = xf ? cid + q : cid + q * R.pitch;
            const int fprev = xf ? fid - R.pitch : fid - 1;
            if (t == 0 || t == 2) v = dmin(v, RDS[fid] > zero ? R.Rp[fid] : R.Rm[fid]);
            else v = dmin(v, RDS[fid] > zero ? R.Rm[fprev] : R.Rp[fprev]);
        }
        if (t == 0 || t == 2) v = dmin(v, NDS[nid] > zero ? N.Rm[nprev] : N.Rp[nprev]);
        else v = dmin(v, NDS[nid] > zero ? N.Rp[nid] : N.Rm[nid]);
        for (int q = 0; q < r; q++) RC[xf ? cid + q : cid + q * R.pitch] = v;
        NC[nid] = v;
    }
}

// Rectangle::getError (Rectangle.cpp:866-890) with ErrorEstimate (Rectangle.hpp:128-130)
// on f slot 1; one flag byte per interior cell, zero outside the tested range.
template <class T>
__global__ void k_flags(const PatchT<T> *patches, const FlagPatch *fps, uint8_t *out) {
    VX_PDL_WAIT();
    const FlagPatch fp = fps[blockIdx.y];
    const PatchT<T> &P = patches[fp.patch];
    const int pit = P.pitch;
    const T *f = P.f1;
    const long long cells = (long long)P.nx * P.np;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cells; c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c / P.np), j = (int)(c - (long long)i * P.np);
        uint8_t flag = 0;
        if (i >= fp.i0 && i < fp.i1 && j >= fp.j0 && j < fp.j1) {
            const T c0 = f[pidx(i, j, pit)];
            const T xp = f[pidx(i + 1, j, pit)], xm = f[pidx(i - 1, j, pit)];
            const T pp = f[pidx(i, j + 1, pit)], pm = f[pidx(i, j - 1, pit)];
            const T two = 2;
            const T e = (T)fp.w[0] * fabs(xp - xm) + (T)fp.w[1] * fabs(pp - pm) + (T)fp.w[2] * fabs(xp - two * c0 + xm) +
                        (T)fp.w[3] * fabs(pp - two * c0 + pm) + (T)fp.w[4] * fabs(c0);
            flag = e > (T)fp.crit ? 1 : 0;
        }
        out[fp.out_off + c] = flag;
    }
}

// Regrid transfer (Rectangle.cpp:892-941, 1100-1128): slots 0 and 1 of the new patch
// from slot 1 of the source.
template <class T>
__global__ void k_xfer(const PatchT<T> *patches, const XferOp *ops, uint8_t *mask) {
    VX_PDL_WAIT();
    const XferOp op = ops[blockIdx.y];
    const PatchT<T> &D = patches[op.dst];
    const PatchT<T> &S = patches[op.src];
    const int w = op.j1 - op.j0;
    const long long cells = (long long)(op.i1 - op.i0) * w;
    const int dpit = D.pitch;
    const int mpit = D.np + 4;  // IndexNS pitch
    uint8_t *m = mask + op.mask_off;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cells; c += (long long)gridDim.x * blockDim.x) {
        const int i = op.i0 + (int)(c / w), j = op.j0 + (int)(c % w);
        if (op.kind == kXferCopy) {
            const int di = i - op.x2, dj = j - op.p2;
            const T v = S.f1[pidx(i - S.x_pos, j - S.p_pos, S.pitch)];
            D.f0[pidx(di, dj, dpit)] = v;
            D.f1[pidx(di, dj, dpit)] = v;
            m[(di + 2) * mpit + (dj + 2)] = 1;
            continue;
        }
        const int r = S.r;
        const int bi = (i - op.x2) * r, bj = (j - op.p2) * r;
        if (op.kind == kXferInterpMissing && m[(bi + 1 + 2) * mpit + (bj + 1 + 2)]) continue;
        T out[kMaxR * kMaxR];
        interp_block(S, S.f1, i - S.x_pos, j - S.p_pos, out);
        for (int k = 0; k < r; k++)
            for (int l = 0; l < r; l++) {
                const int id = pidx(bi + k, bj + l, dpit);
                D.f0[id] = out[l + r * k];
                D.f1[id] = D.f0[id];
                if (op.kind == kXferInterp) m[(bi + k + 2) * mpit + (bj + l + 2)] = 1;
            }
    }
}

void launch_flags(const void *patches, const FlagPatch *fp, int n, uint8_t *out, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) vx_launch(k_flags<float>, dim3(64, n), 256, 0, s, (const PatchT<float> *)patches, fp, out);
    else vx_launch(k_flags<double>, dim3(64, n), 256, 0, s, (const PatchT<double> *)patches, fp, out);
}

void launch_xfer(const void *patches, const XferOp *ops, int n, uint8_t *mask, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) vx_launch(k_xfer<float>, dim3(16, n), 256, 0, s, (const PatchT<float> *)patches, ops, mask);
    else vx_launch(k_xfer<double>, dim3(16, n), 256, 0, s, (const PatchT<double> *)patches, ops, mask);
}

// One block per segment: copy its ops and make their patch ids global to the set.
__device__ __forceinline__ void rebase(GhostOp &op, int b) {
    op.dst += b;
    if (op.src >= 0) op.src += b;
}
__device__ __forceinline__ void rebase(IfaceOp &op, int b) {
    op.coarse += b;
    op.fine += b;
}
__device__ __forceinline__ void rebase(CSyncOp &op, int b) {
    op.nb += b;
    op.caller += b;
}
template <class Op>
__global__ void k_merge_ops(const OpSegment *segs, Op *dst) {
    VX_PDL_WAIT();
    const OpSegment sg = segs[blockIdx.x];
    const Op *src = (const Op *)sg.src;
    for (int k = threadIdx.x; k < sg.count; k += blockDim.x) {
        Op op = src[k];
        rebase(op, sg.base);
        dst[sg.dst_off + k] = op;
    }
}
void merge_ghost_ops(const OpSegment *segs, int nseg, GhostOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch(k_merge_ops<GhostOp>, nseg, 256, 0, s, segs, dst);
}
void merge_iface_ops(const OpSegment *segs, int nseg, IfaceOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch(k_merge_ops<IfaceOp>, nseg, 256, 0, s, segs, dst);
}
void merge_csync_ops(const OpSegment *segs, int nseg, CSyncOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch(k_merge_ops<CSyncOp>, nseg, 256, 0, s, segs, dst);
}

void launch_ghost(const void *patches, const GhostOp *ops, int n, int slot, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) vx_launch(k_ghost<float>, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n, slot);
    else vx_launch(k_ghost<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n, slot);
}

void launch_iface(const void *patches, const IfaceOp *ops, int n, int step, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) vx_launch(k_iface<float>, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n, step);
    else vx_launch(k_iface<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n, step);
}

void launch_csync(const void *patches, const CSyncOp *ops, int n, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) vx_launch(k_csync<float>, (n + 127) / 128, 128, 0, s, (const PatchT<float> *)patches, ops, n);
    else vx_launch(k_csync<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n);
}

}  // namespace vx
