"""Physical constants in the units jclsquant uses (jclsquant/constants.py:1-10)."""
hbar = 6.582e-16  # eV s
kb = 8.617333 * 1e-5  # eV / K
epsilon_0 = 55.26349406e-3  # e^2 / (eV nm)
c = 3e17  # nm / s
e = 1.60217663e-19  # C
hbar_fs = hbar * 1e15  # eV fs
vf_nm_fs = 0.8737422664298289  # nm / fs
a_cc = 0.14199929870718847  # nm
mub_ev_T = 5.7883817982e-5  # eV / T
