// Block-structured AMR on the device: connectivity between patches and the three kinds
// of cross-patch work of one RK stage, each expressed as a list of small operations that
// the device executes in batches.
//
//   ghost fills       Mesh::PushData (Mesh.cpp:91-106 -> Level.cpp:88-151 ->
//                     Rectangle.cpp:307-614, 1130-1214)
//   interface fluxes  coarse faces covered by a finer patch (Rectangle.hpp:132-178,
//                     Rectangle.cpp:1032-1098, 1216-1253)
//   limiter C-sync    Mesh::PushBoundaryC (Mesh.cpp:904-917 -> Rectangle.cpp:1625-1960)
//
// The reference performs these as sequential method calls whose later writes win.  The
// host replays that call sequence into an ordered op list and gives every op the lowest
// batch number that keeps all read-after-write, write-after-read and write-after-write
// orders of the sequence; ops of one batch touch disjoint cells and run in one launch.
#pragma once
#include <cstdint>
#include <vector>

namespace vx {

enum GhostKind : int { kGhostZero = 0, kGhostCopy = 1, kGhostRestrict = 2, kGhostInterp = 3 };

// One ghost/nested cell of patch `dst`.  copy: value of cell (si, sj) of patch `src`;
// restrict: mean of the r x r cells of patch `src` starting at (si, sj); interp: entry
// (sub / r, sub % r) of the conservative 5x5 interpolation around coarse cell (si, sj) of
// patch `src` (Rectangle::GetWenoValueFromCoarseLevel).
struct GhostOp {
    int kind;
    int dst, di, dj;
    int src, si, sj;
    int sub;
};

enum CSyncKind : int { kCSame = 0, kCDiff = 1, kCUpdate = 2 };

// kCSame / kCUpdate: one face k of SetCFromSameLevel / UpdateCFromSameLevel: patch nb's
// face (ni, nj) and the caller's face (ci, cj) (k already added).  kCDiff:
// SetCFromDifferentLevel: coarse face (ni, nj) of patch nb and the caller's r fine faces
// starting at (ci, cj).  t is the reference's orientation argument (0..3).
struct CSyncOp {
    int kind, t;
    int nb, ni, nj;
    int caller, ci, cj;
};

// Coarse face (ci, cj) of patch `coarse` covered by the fine faces starting at (fi, fj)
// of patch `fine` (x faces step in j, p faces step in i).
struct IfaceOp {
    int dir;  // 0: x face, 1: p face
    int coarse, ci, cj;
    int fine, fi, fj;
};

// Error flags of one patch (Rectangle::getError): local cells [i0,i1) x [j0,j1) are
// tested against crit with the patch's five error weights; out_off locates the patch's
// n_x * n_p flag bytes.
struct FlagPatch {
    int patch;
    int i0, i1, j0, j1;
    long long out_off;
    double w[5];
    double crit;
};

// Regrid data transfer (Rectangle.cpp:892-1128) over the cells [i0,i1) x [j0,j1) of the
// source's level (coarse cells for the interpolating kinds): new patch `dst`, source
// patch `src`, (x2, p2) the dst position in source-level cells; mask_off locates dst's
// is_interpolated bytes.
enum XferKind : int { kXferInterp = 0, kXferCopy = 1, kXferInterpMissing = 2 };
struct XferOp {
    int kind, dst, src;
    int i0, i1, j0, j1;
    int x2, p2;
    long long mask_off;
};

struct Batched {
    std::vector<int> ptr;  // batch b = ops[ptr[b] .. ptr[b+1])
};

}  // namespace vx
