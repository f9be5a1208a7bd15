"""Hartree atomic units used by every number on the KMC hot path.

The values and the order in which the derived units are formed follow
PyCD/constants.py:1-45 so that unit conversions round identically: the
precomputed Ewald array, hop rates and residence times are all stated in
atomic units, and parity with the reference depends on the same doubles.
"""

# SI inputs (CODATA 2014, as used by the reference)
EPSILON0 = 8.854187817E-12   # F/m
ANG = 1E-10                  # m
KB = 1.38064852E-23          # J/K
pi = 3.14159265358979323846
EMASS = 9.10938356E-31       # kg
ECHARGE = 1.6021766208E-19   # C
HBAR = 1.054571800E-34       # J s

# derived atomic units
KE = 1 / (4 * pi * EPSILON0)
BOHR = HBAR ** 2 / (EMASS * ECHARGE ** 2 * KE)
HARTREE = HBAR ** 2 / (EMASS * BOHR ** 2)
AUTIME = HBAR / HARTREE
AUTEMPERATURE = HARTREE / KB
AUPOT = HARTREE / ECHARGE

# conversions
EV2J = ECHARGE
ANG2BOHR = ANG / BOHR
ANG2UM = 1.00E-04
ANG2CM = 1.00e-08
J2HARTREE = 1 / HARTREE
SEC2AUTIME = 1 / AUTIME
V2AUPOT = 1 / AUPOT
EV2HARTREE = EV2J * J2HARTREE
SEC2NS = 1.00E+09
SEC2PS = 1.00E+12
SEC2FS = 1.00E+15
K2AUTEMP = 1 / AUTEMPERATURE
AUTIME2NS = SEC2NS / SEC2AUTIME
AUTIME2PS = SEC2PS / SEC2AUTIME
AUTIME2FS = SEC2FS / SEC2AUTIME
BOHR2UM = ANG2UM / ANG2BOHR
BOHR2CM = ANG2CM / ANG2BOHR
