/* A user's problem file written against the C hooks of include/vx.h: the counterpart of
 * the reference's veritas.cpp (initialConditions, settingsOverride, InitialDistribution,
 * GetBY/GetBZ, RefinementOverride), here as plain C functions taking the problem's own
 * parameter block as their `user` pointer.
 *
 * Two mobile species (electrons and ions) in a plasma with a cosine-modulated density
 * and an x-dependent electron drift (f does not factor into x and p parts), vacuum pads
 * beside the domain, a circularly polarised laser whose amplitude rises as sin^2 over
 * `ramp` periods, and a refinement window that flags cells whatever their error. */
#ifndef SIN2_PROBLEM_H_
#define SIN2_PROBLEM_H_

#include <stdint.h>

#include "../../include/vx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sin2_params {
    uint32_t nx, np, Lfinest;  /* base grid (both species), levels */
    double L, pad;              /* domain length and vacuum pad on each side [laser wavelengths] */
    double x_lo, x_hi;          /* plasma edges [wavelengths] */
    double dens, mod_k, mod_amp; /* density / n_c, cos modulation (mode number, amplitude) */
    double Te, Ti, mi;          /* temperatures [keV], ion mass / m_e */
    double pmax_e, pmax_i;      /* momenta in [-pmax, pmax] (m_e c and m_i c) */
    double drift;               /* electron drift amplitude [m_e c], sin(2 pi x / L) */
    double a0, ramp;            /* laser amplitude, sin^2 ramp length [periods] */
    double crit, minEff, sizeWeight, cfl;
    int32_t quadDepth;
    double ref_x0, ref_x1, ref_p; /* RefinementOverride: x in [ref_x0, ref_x1] wavelengths, |p| < ref_p m_e c, electrons */
} sin2_params;

void sin2_defaults(sin2_params *p);
void sin2_initial_conditions(void *user, vx_input *grid, vx_particles *particles, vx_output *output);
void sin2_settings_override(void *user, vx_settings *s);
double sin2_initial_distribution(void *user, const vx_settings *s, double x, double p, int species);
double sin2_get_by(void *user, const vx_settings *s, double x, double t);
double sin2_get_bz(void *user, const vx_settings *s, double x, double t);
int sin2_refinement_override(void *user, const vx_settings *s, double x, double p, int depth, int species);

#ifdef __cplusplus
}
#endif
#endif
