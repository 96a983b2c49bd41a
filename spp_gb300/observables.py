"""Order parameters and pair statistics (the reference's offline analysis,
analyze/analyze.h and analyze/statistics.h, computed from device frames)."""
import ctypes as C
import math

import numpy as np

from . import abi


def order_parameters(p, area):
    """Compute_Order_Parameters (analyze/analyze.h:121-146) of a polarization
    series: mean, error from the autocorrelation length
    (analyze/statistics.h:68-82), sigma2 = variance * area, and both Binder
    forms (binder = 1 - <P^4>/(3<P^2>^2); binder_reference = 1 - <P^4>/(3<P^2>)
    as the reference writes it).  Returns a dict."""
    p = np.ascontiguousarray(p, np.float64)
    out = abi.SppOrderStats()
    abi.check(abi.lib().spp_order_parameters(p.ctypes.data_as(abi._D), len(p), float(area), C.byref(out)),
              "spp_order_parameters")
    return {name: getattr(out, name) for name, _ in abi.SppOrderStats._fields_}


def radial_g(counts, n, L, r_max):
    """g(r) at the bin centres from ordered-pair counts of one frame."""
    counts = np.asarray(counts, np.float64)
    nb = len(counts)
    dr = r_max / nb
    r = (np.arange(nb) + 0.5) * dr
    shell = math.pi * ((np.arange(1, nb + 1) * dr) ** 2 - (np.arange(nb) * dr) ** 2)
    rho = n / (4.0 * L * L)
    return r, counts / (n * rho * shell)


def pair_density(counts, n, lx, ly):
    """Pair_Distribution's normalisation of one frame's counts
    (analyze/analyze.h:411-413): counts / (N * 4 lx ly / (gx gy))."""
    counts = np.asarray(counts, np.float64)
    gx, gy = counts.shape
    return counts / (n * (4.0 * lx * ly / gx / gy))
