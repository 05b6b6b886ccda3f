"""Import the reference's own Python front end with its code-generation deps stubbed.

Test infrastructure only, used in the development container to pin the table
builder and the sparsity of ``pyjac-v2_gb300/mech`` against the reference
itself; it is never imported by the product, by the GPU tests or by the bench
(the reference tree does not exist on the GPU host).

pyJac-v2 imports loopy, pyopencl, cogapp, cgen, yaml, ... at module import
time, although ``mech_interpret.read_mech`` (pyjac/core/mech_interpret.py:106),
``create_jacobian.find_last_species`` (pyjac/core/create_jacobian.py:5131),
``utils.reassign_species_lists`` (pyjac/utils.py:613),
``rate_subs.assign_rates`` (pyjac/core/rate_subs.py:74) and
``create_jacobian.determine_jac_inds`` (pyjac/core/create_jacobian.py:68)
only need numpy.  A ``sys.meta_path`` finder returns mock modules for the
missing packages so that those functions run unmodified.
"""
import importlib.abc
import importlib.machinery
import os
import sys
import types
from unittest import mock

import numpy as np

_STUBS = ("yaml", "loopy", "pytools", "cgen", "cogapp", "cerberus", "pyopencl",
          "codepy", "testconfig", "optionloop", "nose", "tables", "cantera",
          "islpy", "pymbolic", "genpy")


class _Record(object):
    def __init__(self, **kw):
        for k, v in kw.items():
            setattr(self, k, v)

    def copy(self, **kw):
        d = dict(self.__dict__)
        d.update(kw)
        return type(self)(**d)


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        m = mock.MagicMock(name=spec.name)
        m.__path__ = []
        m.__spec__ = spec
        m.__name__ = spec.name
        if spec.name.split(".")[0] == "pytools":
            m.ImmutableRecord = _Record
            m.Record = _Record
            m.UniqueNameGenerator = mock.MagicMock
        if spec.name == "cantera":
            m.__version__ = "2.3.0"
        return m

    def exec_module(self, module):
        pass


class _StubFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        root = fullname.split(".")[0]
        if root in _STUBS:
            return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)
        if fullname == "pyjac.siteconf":
            return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=False)
        return None


_loaded = None


def load(reference="/root/reference"):
    """Return a namespace with the reference's front-end functions."""
    global _loaded
    if _loaded is not None:
        return _loaded
    if not os.path.isdir(os.path.join(reference, "pyjac")):
        raise RuntimeError("reference tree not found at %s" % reference)
    sys.dont_write_bytecode = True
    sys.meta_path.insert(0, _StubFinder())
    if reference not in sys.path:
        sys.path.insert(0, reference)
    site = types.ModuleType("pyjac.siteconf")
    for k in ("CL_INC_DIR", "CL_LIBNAME", "CC_FLAGS", "LDFLAGS", "CL_LIB_DIR",
              "CL_FLAGS", "CL_VERSION", "ADEPT_INC_DIR", "ADEPT_LIB_DIR",
              "ADEPT_LIBNAME"):
        setattr(site, k, [])
    sys.modules["pyjac.siteconf"] = site
    mi = importlib.import_module("pyjac.core.mech_interpret")
    rs = importlib.import_module("pyjac.core.rate_subs")
    cj = importlib.import_module("pyjac.core.create_jacobian")
    ut = importlib.import_module("pyjac.utils")
    en = importlib.import_module("pyjac.core.enum_types")

    # rate_subs.py:314 builds a ragged np.array(cheb_coeff), which numpy>=1.24
    # rejects; fall back to an object array exactly as older numpy did.
    real_array = np.array

    def _array(obj, *a, **kw):
        try:
            return real_array(obj, *a, **kw)
        except ValueError:
            kw.pop("dtype", None)
            return real_array(obj, *a, dtype=object, **kw)

    npmod = types.ModuleType("np_ragged")
    npmod.__dict__.update(np.__dict__)
    npmod.array = _array
    rs.np = npmod

    _loaded = types.SimpleNamespace(read_mech=mi.read_mech,
                                    find_last_species=cj.find_last_species,
                                    reassign_species_lists=ut.reassign_species_lists,
                                    assign_rates=rs.assign_rates,
                                    determine_jac_inds=cj.determine_jac_inds,
                                    RateSpecialization=en.RateSpecialization,
                                    JacobianType=en.JacobianType)
    return _loaded


def reference_tables(mech, therm=None, last_spec=None, rate_spec="hybrid",
                     jac_type="exact", reference="/root/reference"):
    """Run the reference front end on a Chemkin file; return (specs, reacs, val)."""
    ref = load(reference)
    elems, specs, reacs = ref.read_mech(mech, therm)
    specs = ref.find_last_species(specs, last_spec=last_spec)
    ref.reassign_species_lists(reacs, specs)
    val = ref.determine_jac_inds(reacs, specs, getattr(ref.RateSpecialization, rate_spec),
                                 getattr(ref.JacobianType, jac_type))
    return specs, reacs, val
