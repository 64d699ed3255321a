"""Physical constants (jax_cosmo/constants.py:9-27)."""
c = 299792.458  # speed of light [km/s]
tcmb = 2.726  # CMB temperature [K]
rh = 2997.92458  # Hubble radius [Mpc/h]
eta_nu = 0.68130  # neutrino / photon energy density ratio
H0 = 100.0  # Hubble constant [km/s/(Mpc/h)]
C_1 = 5.0 * 1e-14  # intrinsic-alignment normalisation [(h^2 M_sun Mpc^-3)^-1]
rhocrit = 2.7750 * 1e11  # critical density [h^2 M_sun Mpc^-3]
