/* The user problem declared in sin2_problem.h (test fixture: the parity tests load it
 * into the GPU path through vx_run_create_hooks, and the reference build links it behind
 * its own Settings hooks to make the golden states).  Build with -ffp-contract=off. */
#include "sin2_problem.h"

#include <math.h>

static const double kLambda = 1e-6;
static const double kMe = 9.10938291e-31;
static const double kQe = 1.60217657e-19;
static const double kC = 299792458.0;
static const double kEps0 = 8.854187817e-12;
static const double kKeV = 1.602176565e-16;
static const double k2Pi = 6.28318530718;

void sin2_defaults(sin2_params *p) {
    p->nx = 64;
    p->np = 32;
    p->Lfinest = 2;
    p->L = 12.0;
    p->pad = 0.5;
    p->x_lo = 2.0;
    p->x_hi = 10.0;
    p->dens = 0.5;
    p->mod_k = 3.0;
    p->mod_amp = 0.3;
    p->Te = 20.0;
    p->Ti = 5.0;
    p->mi = 16.0;
    p->pmax_e = 1.0;
    p->pmax_i = 0.2;
    p->drift = 0.1;
    p->a0 = 1.5;
    p->ramp = 2.0;
    p->crit = 1e-3;
    p->minEff = 0.8;
    p->sizeWeight = 0.0;
    p->cfl = 0.5;
    p->quadDepth = 2;
    p->ref_x0 = 5.0;
    p->ref_x1 = 6.0;
    p->ref_p = 0.15;
}

void sin2_initial_conditions(void *user, vx_input *grid, vx_particles *particles, vx_output *output) {
    const sin2_params *P = (const sin2_params *)user;
    grid->minEfficiency = P->minEff;
    grid->refinementCriteria = P->crit;
    grid->cfl = P->cfl;
    grid->sizeWeight = P->sizeWeight;
    grid->preLength = P->pad * kLambda;
    grid->postLength = P->pad * kLambda;
    grid->nx = P->nx;
    grid->r = 2;
    grid->Lfinest = P->Lfinest;
    grid->plasma_xl_bound = P->x_lo * kLambda;
    grid->plasma_xr_bound = P->x_hi * kLambda;
    grid->ntempEM = 1;
    grid->tempEM[0] = 0.0;
    particles->nspecies = 2;
    particles->mass[0] = kMe;
    particles->charge[0] = -kQe;
    particles->mass[1] = P->mi * kMe;
    particles->charge[1] = kQe;
    for (int s = 0; s < 2; s++) {
        particles->np[s] = P->np;
        particles->dp[s] = 0.1;
        particles->pmin[s] = 0.1;
        particles->nmisc[s] = 2;
        particles->misc[s][0] = 0.0;
        particles->misc[s][1] = 0.0;
    }
    output->time = output->rectangleData = output->charge = output->energy = output->potential = 0;
    output->EFieldLongitudinal = output->EFieldTransverse = output->BFieldTransverse = output->AFieldSquared = 0;
    output->precision = 15;
}

/* dp and pmin from the momentum ranges; temp[s] = {n0, sigma (kg^2 m^2 / s^2)}, tempEM =
 * {lambda, B amplitude}. */
void sin2_settings_override(void *user, vx_settings *s) {
    const sin2_params *P = (const sin2_params *)user;
    const double pm[2] = {P->pmax_e, P->pmax_i};
    const double T[2] = {P->Te, P->Ti};
    s->dx = P->L * kLambda / s->x_size;
    s->quadratureDepth = P->quadDepth;
    const double omega = k2Pi * kC / kLambda;
    const double nc = omega * omega * s->m[0] * kEps0 / (s->q[0] * s->q[0]);
    for (int i = 0; i < 2; i++) {
        const double mc = s->m[i] * kC;
        s->dp[i] = 2.0 * pm[i] * mc / s->p_size[i];
        s->pmin[i] = -pm[i] * mc;
        s->ntemp[i] = 2;
        s->temp[i][0] = P->dens * nc;
        s->temp[i][1] = s->m[i] * (T[i] * kKeV);
    }
    s->ntempEM = 2;
    s->tempEM[0] = kLambda;
    s->tempEM[1] = P->a0 * s->m[0] * kC / fabs(s->q[0]) * (k2Pi / kLambda);
}

double sin2_initial_distribution(void *user, const vx_settings *s, double x, double p, int species) {
    const sin2_params *P = (const sin2_params *)user;
    if (!(x > s->plasma_xl_bound && x < s->plasma_xr_bound)) return 0.0;
    const double xl = x / kLambda;
    const double n = s->temp[species][0] * (1.0 + P->mod_amp * cos(k2Pi * P->mod_k * xl / P->L));
    const double sig = s->temp[species][1];
    double u = p;
    if (species == 0) u = p - P->drift * s->m[0] * kC * sin(k2Pi * xl / P->L);
    return n * exp(-(u * u) / (2.0 * sig)) / sqrt(k2Pi * sig);
}

/* Envelope sin^2(pi tau / (2 ramp T)) up to tau = ramp T, then 1; tau = t - x / c. */
static double envelope(double tau, double ramp_T, double *deriv) {
    if (tau <= 0.0) {
        *deriv = 0.0;
        return 0.0;
    }
    if (tau >= ramp_T) {
        *deriv = 0.0;
        return 1.0;
    }
    const double a = 0.5 * k2Pi / (2.0 * ramp_T);
    const double sn = sin(a * tau), cs = cos(a * tau);
    *deriv = 2.0 * a * sn * cs;
    return sn * sn;
}

/* A = (A0/k) g(tau) (cos(w tau), sin(w tau)) in (y, z): B_y = -dA_z/dx, B_z = dA_y/dx. */
double sin2_get_by(void *user, const vx_settings *s, double x, double t) {
    const sin2_params *P = (const sin2_params *)user;
    const double k = k2Pi / s->tempEM[0], w = kC * k, T = s->tempEM[0] / kC;
    const double tau = t - x / kC;
    double dg;
    const double g = envelope(tau, P->ramp * T, &dg);
    /* dA_z/dx = -(1/c) d/dtau [g sin(w tau)] (A0/k) */
    const double dAz = -(s->tempEM[1] / k) / kC * (dg * sin(w * tau) + g * w * cos(w * tau));
    return -dAz;
}

double sin2_get_bz(void *user, const vx_settings *s, double x, double t) {
    const sin2_params *P = (const sin2_params *)user;
    const double k = k2Pi / s->tempEM[0], w = kC * k, T = s->tempEM[0] / kC;
    const double tau = t - x / kC;
    double dg;
    const double g = envelope(tau, P->ramp * T, &dg);
    const double dAy = -(s->tempEM[1] / k) / kC * (dg * cos(w * tau) - g * w * sin(w * tau));
    return dAy;
}

int sin2_refinement_override(void *user, const vx_settings *s, double x, double p, int depth, int species) {
    const sin2_params *P = (const sin2_params *)user;
    (void)depth;
    if (species != 0) return 0;
    const double xl = x / kLambda;
    return xl >= P->ref_x0 && xl <= P->ref_x1 && fabs(p) < P->ref_p * s->m[0] * kC;
}
