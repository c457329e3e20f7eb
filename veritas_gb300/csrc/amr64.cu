// Device execution of the AMR op lists built in amr.cpp.  Each launch runs one batch of
// ops that touch disjoint cells; the batches run in order on the context stream.
// Compiled with --fmad=false: every expression keeps the reference's operation order.
// The op kernels here serve FP64 patches (the FP32 precision form's are in stage32.cu,
// over the same bodies); the flagging and regrid transfer kernels serve both.
#include <cuda_runtime.h>

#include "amr_ops.cuh"

namespace vx {

template <class T>
__global__ void k_ghost(const PatchT<T> *patches, const GhostOp *ops, int n, int slot) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) ghost_op(patches, ops, k, slot);
}
template <class T>
__global__ void k_iface(const PatchT<T> *patches, const IfaceOp *ops, int n, int step) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) iface_op(patches, ops, k, step);
}
template <class T>
__global__ void k_csync(const PatchT<T> *patches, const CSyncOp *ops, int n) {
    VX_PDL_WAIT();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) csync_op(patches, ops, k);
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
// Blocks (segment, part): part y of gridDim.y copies every gridDim.y-th stretch of 256 ops,
// so that a long segment is not left to one block.
template <class Op>
__global__ void k_merge_ops(const OpSegment *segs, Op *dst) {
    VX_PDL_WAIT();
    const OpSegment sg = segs[blockIdx.x];
    const Op *src = (const Op *)sg.src;
    for (int k = blockIdx.y * blockDim.x + threadIdx.x; k < sg.count; k += gridDim.y * blockDim.x) {
        Op op = src[k];
        rebase(op, sg.base);
        dst[sg.dst_off + k] = op;
    }
}
constexpr int kMergeParts = 8;
void merge_ghost_ops(const OpSegment *segs, int nseg, GhostOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch_plain(k_merge_ops<GhostOp>, dim3(nseg, kMergeParts), 256, 0, s, segs, dst);
}
void merge_iface_ops(const OpSegment *segs, int nseg, IfaceOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch_plain(k_merge_ops<IfaceOp>, dim3(nseg, kMergeParts), 256, 0, s, segs, dst);
}
void merge_csync_ops(const OpSegment *segs, int nseg, CSyncOp *dst, cudaStream_t s) {
    if (nseg > 0) vx_launch_plain(k_merge_ops<CSyncOp>, dim3(nseg, kMergeParts), 256, 0, s, segs, dst);
}

// Host tables to the device through the SMs: page-locked host memory read over the
// host link, so the copy does not queue on a copy engine behind other threads' transfers.
__global__ void k_copy_from_host(const uint4 *src, uint4 *dst, size_t n16) {
    VX_PDL_WAIT();
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
void copy_from_host(const void *src_dev, void *dst, size_t bytes, cudaStream_t s) {
    const size_t n16 = bytes / 16;
    if (n16 == 0) return;
    const int blocks = (int)std::min<size_t>((n16 + 255) / 256, 1024);
    vx_launch_plain(k_copy_from_host, blocks, 256, 0, s, (const uint4 *)src_dev, (uint4 *)dst, n16);
}

void launch_ghost(const void *patches, const GhostOp *ops, int n, int slot, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) launch_ghost32(patches, ops, n, slot, s);
    else vx_launch(k_ghost<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n, slot);
}

void launch_iface(const void *patches, const IfaceOp *ops, int n, int step, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) launch_iface32(patches, ops, n, step, s);
    else vx_launch(k_iface<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n, step);
}

void launch_csync(const void *patches, const CSyncOp *ops, int n, int prec, cudaStream_t s) {
    if (n <= 0) return;
    if (prec == kF32) launch_csync32(patches, ops, n, s);
    else vx_launch(k_csync<double>, (n + 127) / 128, 128, 0, s, (const PatchT<double> *)patches, ops, n);
}

}  // namespace vx
