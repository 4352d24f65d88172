"""Physical constants and unit factors of the e-ph vertex path.

Values follow elphbolt's ``src/params.f90:27-57`` exactly, so that every unit
conversion (Ry -> eV, Rydberg mass -> amu, 2*pi/hbar in eV.ps) agrees bit for
bit with the reference's double-precision parameters.  The C++/CUDA side
defines the same numbers in ``csrc/ephg_common.cuh``.
"""
import math

qe = 1.602176634e-19          # C
me = 9.1093837015e-31         # kg
amu = 1.66053906660e-27       # kg
hbar = 1.05457172647e-22      # J.ps
hbar_eVps = hbar / qe         # eV.ps
kB = 1.380649e-23 / qe        # eV/K
pi = 4.0 * math.atan(1.0)
twopi = 2.0 * pi

Hartree2radTHz = 27.2116 * qe / hbar
Hartree2eV = 27.2116
Ryd2radTHz = 0.5 * Hartree2radTHz
Ryd2eV = 0.5 * Hartree2eV
Ryd2meV = Ryd2eV * 1.0e3
Ryd2amu = 2.0 * me / amu
bohr2nm = 0.052917721092

# |g|^2 unit factor of wannier.f90:923
g2unitfactor = Ryd2eV ** 3 * Ryd2amu
