// Shared host/device definitions for the Veritas GB300 path.
//
// Phase-space patches ("Rectangles", Rectangle.hpp:6-80 in Veritas) live in HBM as
// structure-of-arrays blocks.  Every per-patch array has (n_x+4) rows of `pitch`
// doubles (or floats); row r holds x-index i = r-2, column c holds p-index j = c-2, so
// p is the fast, coalesced axis exactly as in the reference's IndexNS(i,j)
// (Rectangle.hpp:106), but each f slot, flux and limiter array is its own plane instead
// of the reference's interleaved Index3/Index6 records.
#pragma once
#include <cstdint>

#ifndef VX_HD
#ifdef __CUDACC__
#define VX_HD __host__ __device__
#else
#define VX_HD
#endif
#endif

namespace vx {

// Physical constants exactly as the reference defines them (veritas.hpp:22-30).
constexpr double kEps0Inv = 1.1294e+11;
constexpr double kEps0 = 8.854187817e-12;
constexpr double kMuInv = 795774.715482;
constexpr double kCs = 299792458.0;
constexpr double kCInv = 3.33564095e-9;
constexpr double kDPI = 6.28318530718;

// Low-storage description of the 6-stage Runge-Kutta tableau (Rectangle.cpp:1396-1517,
// EMSolver.cpp:204-338).  Row s holds a_{s,0..s}; row 5 holds the b weights.
constexpr double kRK[6][6] = {
    {0.5, 0, 0, 0, 0, 0},
    {0.221776, 0.110224, 0, 0, 0, 0},
    {-0.04884659515311857, -0.17772065232640102, 0.8465672474795197, 0, 0, 0},
    {-0.15541685842491548, -0.3567050098221991, 1.0587258798684427, 0.30339598837867193, 0, 0},
    {0.2014243506726763, 0.008742057842904185, 0.15993995707168115, 0.4038290605220775, 0.22606457389066084, 0},
    {0.15791629516167136, 0.0, 0.18675894052400077, 0.6805652953093346, -0.27524053099500667, 0.25},
};

enum Precision : int { kF64 = 64, kF32 = 32 };
// Poisson solver: the reference's LU in its rounding order, or the O(n) prefix-scan solve
enum PoissonSolver : int { kPoissonLU = 0, kPoissonScan = 1 };

// Device view of one patch.  T is the storage type of f / fluxes / limiter planes.
template <class T>
struct PatchT {
    int nx, np, x_pos, p_pos;
    int depth, rtb;         // rtb = r^depth (Rectangle::relativeToBottom)
    int pitch;              // row pitch in elements
    int xm, xp, pm, pp;     // active face window [xm,xp) x [pm,pp) (Rectangle.cpp:1257-1261)
    int run, species;
    int has_iface;          // any coarse/fine interface face on this patch
    int r;                  // refinement ratio
    double dx, dp, dx_inv, dp_inv;
    double pmin, q, qq, mass, cc, g2;  // qq=q*q, cc=cs*cs*m, g2=(m_inv*c_inv)^2
    // FP32 precision form: f is stored as f * fnorm; pnorm = 1/(m c) makes momenta
    // dimensionless (dpn = dp * pnorm); kx = c^2 m / dp and kp = c^2 m / dx scale the
    // rationalised Lorentz-factor differences into face velocities; weno_eps is the WENO
    // regulariser in the scaled units.
    double fnorm, pnorm, dpn, kx, kp;
    float weno_eps;
    // FP32 copies of the scalars the FP32 kernels use (no FP64 arithmetic in their
    // loops): p_min / (m c), dp / (m c), kx, kp, 1/dx, 1/dp, q, q^2 / (m c)^2
    float pminf, dpnf, kxf, kpf, dxif, dpif, qf, a2nf;
    // FP32 moments: final scales of the rho and J column sums (1/fnorm folded in)
    double msc_rho, msc_j;
    T *f0, *f1, *f2;
    T *gam;                 // gamma at (x-face i, p-face j), i in [-1,nx+1], j in [-1,np+1]
    T *ex, *fx, *ep, *fp;   // face velocities and reconstructed face values
    T *FxH[6], *FpH[6];     // high-order flux history, one plane per RK stage
    T *FxL, *FpL;           // stage-0 low-order fluxes
    T *FxDS, *FpDS;         // antidiffusive stage fluxes
    T *Rp, *Rm, *Cx, *Cp;   // Zalesak limiter
    uint8_t *nested;        // is_nested (cells covered by a finer patch)
    uint8_t *ifx, *ifp;     // is_interrior_level_boundary_x / _p
    double *chargeR, *currentR;  // per finest column of this patch (n_x * rtb)
    const double *relc;     // interpolation weights onto the rtb finest sub-cells, 3*rtb
    const double *refc;     // interpolation weights onto the r sub-cells of a coarse cell, 3*r
    const float *relc32;    // FP32 relc, then the three weights summed over the sub-cells
};

// Per-run field block on the device (EMSolver state, EMSolver.hpp:9-49).
struct RunFields {
    int n;              // x_size_finest
    int pre, post;      // vacuum pads
    int nf;             // n + pre + post
    double dx0;         // finest dx
    double *By, *Bz, *Ey, *Ez, *Ay, *Az;  // 8 slots each, slot-major: [slot*nf + i]
    double *asq;        // a_squared, n+1 (last entry stays 0)
    double *phi;        // n
    double *charge, *J, *neut;  // n
    double *efin;       // E_x at finest cells, n (recomputed after every Poisson solve)
    double *ex0;        // scalar
    float *acell32;     // FP32 Ay^2 + Az^2 (slot 1) at every cell of the field grid, nf
    float *asq32;       // FP32 copies of asq (n+1) and efin (n) for the FP32 form
    float *efin32;
};

VX_HD inline int pidx(int i, int j, int pitch) { return (i + 2) * pitch + (j + 2); }

}  // namespace vx
