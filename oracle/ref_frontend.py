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


class _LoopyArg(object):
    """Stand-in for loopy's kernel-argument classes (ArrayArg, ValueArg,
    TemporaryVariable ...): keeps the name and keyword arguments, so that the
    reference's array creator (pyjac/core/array_creator.py creator.__call__
    :1588-1656) builds real access strings such as 'Pr[j, i + 4]'."""

    def __init__(self, name, *args, **kw):
        self.name = name
        self._kw = dict(kw)
        self.__dict__.update(kw)

    def copy(self, **kw):
        d = dict(self._kw)
        d.update(kw)
        return _LoopyArg(d.pop("name", self.name), **d)


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        m = mock.MagicMock(name=spec.name)
        m.__path__ = []
        m.__spec__ = spec
        m.__name__ = spec.name
        if spec.name == "loopy":
            for k in ("ArrayArg", "GlobalArg", "TemporaryVariable", "ValueArg", "ConstantArg"):
                setattr(m, k, _LoopyArg)
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


def load(reference=None):
    """Return a namespace with the reference's front-end functions, imported
    from the tree at `reference` (default: the PYJAC_REFERENCE environment
    variable)."""
    global _loaded
    if _loaded is not None:
        return _loaded
    reference = reference or os.environ.get("PYJAC_REFERENCE")
    if not reference or not os.path.isdir(os.path.join(reference, "pyjac")):
        raise RuntimeError("reference tree not found (%r); set PYJAC_REFERENCE" % reference)
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
    # array_creator.py:2354 uses np.in1d, which numpy 2 removed (np.isin is
    # the same function)
    arc = importlib.import_module("pyjac.core.array_creator")
    npc = types.ModuleType("np_in1d")
    npc.__dict__.update(np.__dict__)
    npc.in1d = np.isin
    arc.np = npc

    _loaded = types.SimpleNamespace(read_mech=mi.read_mech,
                                    find_last_species=cj.find_last_species,
                                    reassign_species_lists=ut.reassign_species_lists,
                                    assign_rates=rs.assign_rates,
                                    determine_jac_inds=cj.determine_jac_inds,
                                    RateSpecialization=en.RateSpecialization,
                                    JacobianType=en.JacobianType,
                                    rate_subs=rs, array_creator=arc,
                                    loopy_utils=importlib.import_module(
                                        "pyjac.loopy_utils.loopy_utils"))
    return _loaded


def reference_tables(mech, therm=None, last_spec=None, rate_spec="hybrid",
                     jac_type="exact", reference=None):
    """Run the reference front end on a Chemkin file; return (specs, reacs, val)."""
    ref = load(reference)
    elems, specs, reacs = ref.read_mech(mech, therm)
    specs = ref.find_last_species(specs, last_spec=last_spec)
    ref.reassign_species_lists(reacs, specs)
    val = ref.determine_jac_inds(reacs, specs, getattr(ref.RateSpecialization, rate_spec),
                                 getattr(ref.JacobianType, jac_type))
    return specs, reacs, val


def reference_rate_kernels(mech, therm=None, conp=True, reference=None, test_size=16):
    """The reference's own instruction text of the species-rate sub-kernels
    whose forms no shipped kernel exercises, generated by its generators
    (pyjac/core/rate_subs.py) for a Chemkin file, C language, C order,
    hybrid rate specialisation: {name: knl_info} for 'plog'
    (get_plog_arrhenius_rates :2084), 'cheb' (get_cheb_arrhenius_rates
    :1904), 'sri' (get_sri_kernel :2472), 'troe' (get_troe_kernel :2350),
    'extra_var' (get_extra_var_rates :798) and 'temperature'
    (get_temperature_rate :963), and the reference's rate tables."""
    ref = load(reference)
    rs, arc, lu = ref.rate_subs, ref.array_creator, ref.loopy_utils
    elems, specs, reacs = ref.read_mech(mech, therm)
    specs = ref.find_last_species(specs)
    ref.reassign_species_lists(reacs, specs)
    spec = ref.RateSpecialization.hybrid
    opts = lu.loopy_options(width=None, depth=None, lang="c", order="C", rate_spec=spec)
    info = rs.assign_rates(reacs, specs, spec)
    nst = arc.NameStore(opts, info, conp, test_size)
    out = {}
    if info["plog"]["num"]:
        out["plog"] = rs.get_plog_arrhenius_rates(opts, nst, info["plog"]["max_P"], test_size=test_size)
    if info["cheb"]["num"]:
        out["cheb"] = rs.get_cheb_arrhenius_rates(opts, nst, np.max(info["cheb"]["num_P"]),
                                                  np.max(info["cheb"]["num_T"]), test_size=test_size)
    for name, fn in (("sri", rs.get_sri_kernel), ("troe", rs.get_troe_kernel)):
        k = fn(opts, nst, test_size=test_size)
        if k:
            out[name] = k
    out["extra_var"] = rs.get_extra_var_rates(opts, nst, conp=conp, test_size=test_size)
    out["temperature"] = rs.get_temperature_rate(opts, nst, conp=conp, test_size=test_size)
    for k, v in list(out.items()):
        out[k] = v[0] if isinstance(v, list) else v
    return out, info, specs
