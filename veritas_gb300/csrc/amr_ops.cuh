// Device bodies of the AMR op batches built in amr.cpp (ghost fills, coarse/fine
// interface fluxes, limiter coefficient exchange; one op per call) and the coarse-level
// interpolation, shared by amr64.cu (FP64 patches, compiled without contraction, so every
// expression keeps the reference's operation order) and stage32.cu (FP32 patches of the
// precision form).
#pragma once
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
__device__ __forceinline__ void ghost_op(const PatchT<T> *patches, const GhostOp *ops, int k, int slot) {
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
__device__ __forceinline__ void iface_op(const PatchT<T> *patches, const IfaceOp *ops, int k, int step) {
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
__device__ __forceinline__ void csync_op(const PatchT<T> *patches, const CSyncOp *ops, int k) {
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

}  // namespace vx
