"""pyjac-v2_gb300: GB300-native batched species rates and analytical Jacobians.

A drop-in for pyJac-v2's generated ``species_rates`` / ``jacobian`` path:
the Chemkin front end and pyJac's data conventions are kept
(phi = (T, V or P, n_0 .. n_{Ns-2}), data order C or F, Jacobian full or
sparse CRS/CCS), and the evaluation runs in hand-written FP64 CUDA kernels for
sm_103a behind a C ABI (``include/pyjac_gb300.h``).

The package directory name contains a hyphen, so import it with
``importlib.import_module("pyjac-v2_gb300")``.
"""
from .mech import Mechanism, load_mechanism, ChemkinError  # noqa: F401

__version__ = "0.1.0"
