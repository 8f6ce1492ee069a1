from scipy.special import erf, erfc  # noqa: F401
