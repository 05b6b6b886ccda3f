"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU.

The oracle (oracle/) is imported here only as the checker.
"""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DATA = os.path.join(ROOT, "data")
GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference tree, for the live front-end check (skipped when unset)
REFERENCE = os.environ.get("PYJAC_REFERENCE", "")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pkg(sub=None):
    return importlib.import_module("pyjac-v2_gb300" + ("." + sub if sub else ""))


def oracle_mod():
    return importlib.import_module("oracle")


MECH_FILES = {
    "h2o2": (os.path.join(DATA, "h2o2.inp"), None),
    "gri30": (os.path.join(DATA, "grimech30.inp"), os.path.join(DATA, "thermo30.dat")),
    "testmech": (os.path.join(GOLDEN, "test_mech.inp"), None),
}

_cache = {}


def load_mech(name, jac_type="exact"):
    """Mechanism by name; jac_type 'approximate' gives the tables of that
    Jacobian type (pattern without the bath-gas full rows)."""
    if jac_type != "exact":
        key = (name, jac_type)
        if key not in _cache:
            base = load_mech(name)
            _cache[key] = pkg("mech").Mechanism(base.elements, base.species, base.reactions,
                                                base.rate_spec, jac_type, source=base.source)
        return _cache[key]
    if name not in _cache:
        if name == "synthetic500":
            # the 500-species, 2,500-reaction benchmark mechanism (seed 0),
            # generated once per machine outside the repository
            import tempfile
            syn = pkg("mech.synthetic")
            path = os.path.join(tempfile.gettempdir(), "pyjac_gb300_synthetic500_seed0.inp")
            if not os.path.exists(path):
                syn.write(path + ".tmp")
                os.replace(path + ".tmp", path)
            _cache[name] = pkg().load_mechanism(path)
        elif name == "synthetic_small":
            syn = pkg("mech.synthetic")
            path = os.path.join(GOLDEN, "synthetic_small.inp")
            if not os.path.exists(path):
                syn.write(path, **SYNTHETIC_SMALL)
            _cache[name] = pkg().load_mechanism(path)
        else:
            mech, therm = MECH_FILES[name]
            _cache[name] = pkg().load_mechanism(mech, therm)
    return _cache[name]


# small all-forms synthetic mechanism used by parity tests (seeded, deterministic)
SYNTHETIC_SMALL = dict(n_species=40, n_reactions=120, seed=3, frac_thd=0.15, frac_troe=0.15,
                       frac_sri=0.1, frac_plog=0.1, frac_cheb=0.1)


def bath_rich_states(mech, n, seed, conp=True, x_floor=1e-6):
    """Seeded states whose bath gas holds half the mixture (finite-difference friendly)."""
    states = pkg("states")
    P, phi = states.draw_states(mech.n_species, n, seed=seed, x_floor=x_floor, conp=conp)
    T = phi[:, 0]
    Pr = P if conp else phi[:, 1]
    V = phi[:, 1] if conp else P
    ntot = Pr * V / (8314.4621 * T)
    phi[:, 2:] *= 0.5 * ntot[:, None] / phi[:, 2:].sum(axis=1, keepdims=True)
    return P, phi


def row_rel_err(J, Jref):
    """max |J - Jref| / max_row |Jref| over all entries (dense, (n, NN, NN))."""
    scale = np.abs(Jref).max(axis=-1, keepdims=True)
    scale[scale == 0] = 1.0
    return float((np.abs(J - Jref) / scale).max())


def rel_err(a, b, floor=1e-300):
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
