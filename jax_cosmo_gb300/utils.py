"""Scale factor / redshift conversions (jax_cosmo/utils.py:2-9)."""


def z2a(z):
    """converts from redshift to scale factor"""
    return 1.0 / (1.0 + z)


def a2z(a):
    """converts from scale factor to redshift"""
    return 1.0 / a - 1.0
