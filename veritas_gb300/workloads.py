"""The laser / plasma workloads the benchmark times and the full-size parity tests run.

All three are the built-in laser / plasma-slab problem (x in [0, 100] laser wavelengths,
p in [-2, 2] m_e c, a slab with 5-wavelength linear ramps on [15, 20] and [80, 85], a
Gaussian-envelope pulse of FWHM 10 periods injected at x = 0, CFL 0.5):

* ``laser_slab_2048x256``: one level, 2048 x 256, 0.01 n_c, T = 1 keV, a0 = 1.
* ``laser_slab_amr_4096x512``: base 4096 x 512, two levels with refinement ratio 2,
  refinement criterion 1e-6 of the peak of f (size weight 1).
* ``laser_wakefield_amr_16384x1024``: base 16384 x 1024, three levels, 0.005 n_c,
  a0 = 2, T = 0.5 keV.
"""
from __future__ import annotations

import dataclasses

from . import Problem


def laser_slab_2048x256(**over) -> Problem:
    p = Problem(L=100.0, nx=2048, np=256, Lfinest=1, pmax=2.0, dens=0.01, x1=15, x2=20, x3=80, x4=85, Te=1.0,
                a0=1.0, fwhm=10.0, delay=10.0, cfl=0.5, quadDepth=2, precision=64)
    return dataclasses.replace(p, **over)


def laser_slab_amr_4096x512(**over) -> Problem:
    p = laser_slab_2048x256()
    p.nx, p.np, p.Lfinest, p.r = 4096, 512, 2, 2
    p.crit, p.sizeWeight = 1e-6, 1.0
    return dataclasses.replace(p, **over)


def laser_wakefield_amr_16384x1024(**over) -> Problem:
    p = laser_slab_2048x256()
    p.nx, p.np, p.Lfinest, p.r = 16384, 1024, 3, 2
    p.dens, p.a0, p.Te = 0.005, 2.0, 0.5
    p.crit, p.sizeWeight = 1e-6, 1.0
    return dataclasses.replace(p, **over)


WORKLOADS = {
    "laser_slab_2048x256": laser_slab_2048x256,
    "laser_slab_amr_4096x512": laser_slab_amr_4096x512,
    "laser_wakefield_amr_16384x1024": laser_wakefield_amr_16384x1024,
}
