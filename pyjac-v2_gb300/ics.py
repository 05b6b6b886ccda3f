"""Binary initial-condition files (the reference's read_initial_conditions,
pyjac/kernel_utils/common/read_initial_conditions.cpp.in:30-116), through the
library's C entry points.

One record of NN + 1 doubles per state, C order on disk:
[T, param, phi_1 (extra variable), n_0 .. n_{Ns-2}], param = P for constant
pressure and V for constant volume.
"""
import os

import numpy as np

from . import _lib


def read_initial_conditions(path, n, nn, order="C"):
    """Return (param (n,), phi) with phi (n, nn) for order 'C', (nn, n) for 'F'."""
    param = np.empty(int(n))
    phi = np.empty((int(n), int(nn)) if order == "C" else (int(nn), int(n)))
    _lib.check("pjg_read_initial_conditions", _lib.load().pjg_read_initial_conditions(
        os.fsencode(path), int(n), int(nn), order.encode(), param.ctypes.data, phi.ctypes.data))
    return param, phi


def write_initial_conditions(path, param, phi, order="C"):
    """Write param (n,) and phi ((n, nn) for 'C', (nn, n) for 'F') as records."""
    param = np.ascontiguousarray(param, dtype=np.float64)
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    n = param.size
    if phi.size % max(n, 1):
        raise ValueError("phi must hold n x nn values")
    nn = phi.size // n if n else 2
    _lib.check("pjg_write_initial_conditions", _lib.load().pjg_write_initial_conditions(
        os.fsencode(path), n, nn, order.encode(), param.ctypes.data, phi.ctypes.data))
