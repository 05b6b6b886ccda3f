"""Python API over the C ABI.

Two layers:

* :class:`Evaluator` — device-pointer evaluation on torch CUDA tensors
  (asynchronous on the current torch stream).  This is what the torch
  ``autograd.Function`` and the benchmarks use.
* :func:`pywrap` — a module-like object exposing ``PyJacobianKernel`` and
  ``PySpecies_RatesKernel`` with the call signatures of pyJac's generated
  Cython wrapper (pyjac/pywrap/pyjacob_wrapper.pyx.in:19-92):
  ``Py<Name>Kernel(problem_size, work_size, do_not_compile=False)``,
  ``species_names()``, ``reaction_strings()``, ``num_reactions()``,
  ``num_species()``, ``required_working_memory()``, ``resize(...)`` and
  ``__call__(param, phi, out)`` on float64 numpy arrays in the kernel's data
  order.  Arguments follow pywrap_gen.py:175-205 (Jacobian: param, phi, jac;
  species rates: P_arr, phi, dphi).
"""
import ctypes
import types

import numpy as np

from . import _lib
from .pack import PackedTables

KIND_RATES, KIND_JAC = 0, 1
_FORMATS = {"full": 0, "sparse": 1}


def _fmt(jac_format):
    if isinstance(jac_format, str):
        if jac_format not in _FORMATS:
            raise ValueError("jac_format must be 'full' or 'sparse'")
        return _FORMATS[jac_format]
    return int(jac_format)


def _order(order):
    if order not in ("C", "F"):
        raise ValueError("order must be 'C' or 'F'")
    return order.encode()


def _tables_struct(pk):
    """The pjg_tables struct over a PackedTables' arrays (which must outlive it)."""
    t = _lib.PjgTables()
    t.ns, t.nr, t.flags = pk.ns, pk.nr, pk.flags
    t.rxn = pk.rxn.ctypes.data
    t.species = pk.species.ctypes.data_as(_lib._DP)
    t.thd_spec = pk.thd_spec.ctypes.data_as(_lib._I32P)
    t.thd_coef = pk.thd_coef.ctypes.data_as(_lib._DP)
    t.n_thd = pk.n_thd
    t.aux = pk.aux.ctypes.data_as(_lib._DP)
    t.n_aux = pk.n_aux
    t.nnz = pk.nnz
    t.crs_row_ptr = pk.crs_row_ptr.ctypes.data_as(_lib._I32P)
    t.crs_col_ind = pk.crs_col_ind.ctypes.data_as(_lib._I32P)
    t.ccs_col_ptr = pk.ccs_col_ptr.ctypes.data_as(_lib._I32P)
    t.ccs_row_ind = pk.ccs_row_ind.ctypes.data_as(_lib._I32P)
    return t


def reaction_order(mech, with_flags=False):
    """The order in which the device tables hold the mechanism's reactions,
    computed on the host (pjg_reaction_order, no device needed): arrays
    (orig, cls) with orig[p] the mechanism index of packed record p and cls[p]
    the code that evaluates it (0 the elementary class A + B <=> C + D, 1..10
    the mass-action patterns, 11..13 the third-body and fall-off patterns, -1
    the general code).  with_flags=True adds the packed records' flag words
    (the packing's [M]-reuse marks RX_SAMEM = 1 << 20, RX_SAMELNM = 1 << 21
    included)."""
    pk = PackedTables(mech)
    t = _tables_struct(pk)
    orig = np.zeros(pk.nr, dtype=np.int32)
    cls = np.zeros(pk.nr, dtype=np.int32)
    flags = np.zeros(pk.nr, dtype=np.int32)
    _lib.check("pjg_reaction_order", _lib.load().pjg_reaction_order(
        ctypes.byref(t), orig.ctypes.data_as(_lib._I32P), cls.ctypes.data_as(_lib._I32P),
        flags.ctypes.data_as(_lib._I32P)))
    return (orig, cls, flags) if with_flags else (orig, cls)


class DeviceMechanism(object):
    """Mechanism tables uploaded to the current CUDA device (owns a pjg_mech)."""

    def __init__(self, mech):
        lib = _lib.load()
        self.mech = mech
        self.packed = pk = PackedTables(mech)
        t = _tables_struct(pk)
        h = ctypes.c_void_p()
        _lib.check("pjg_mech_create", lib.pjg_mech_create(ctypes.byref(t), ctypes.byref(h)))
        self.handle = h
        self._lib = lib

    def close(self):
        if getattr(self, "handle", None) and self.handle.value:
            self._lib.pjg_mech_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nn(self):
        return self.mech.nn

    @property
    def nnz(self):
        return self.packed.nnz

    def jacobian_indices(self, order="C"):
        n = ctypes.c_int32()
        ptr = np.zeros(self.nn + 1, dtype=np.int32)
        ind = np.zeros(self.nnz, dtype=np.int32)
        _lib.check("pjg_jacobian_indices", self._lib.pjg_jacobian_indices(
            self.handle, _order(order), ptr.ctypes.data_as(_lib._I32P),
            ind.ctypes.data_as(_lib._I32P), ctypes.byref(n)))
        return ptr, ind


class Evaluator(DeviceMechanism):
    """Species rates / Jacobian / J^T v on torch CUDA float64 tensors.

    Shapes: order 'C' — phi (N, NN); order 'F' — phi (NN, N).  Outputs have the
    matching layout: dphi like phi; dense jac (N, NN, NN) for 'C' and
    (NN, NN, N) [col, row, state] for 'F'; sparse jac (N, nnz) / (nnz, N).
    """

    def _prep(self, param, phi, order):
        import torch
        for x in (param, phi):
            if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == torch.float64):
                raise TypeError("expected CUDA float64 tensors")
            if not x.is_contiguous():
                raise ValueError("tensors must be contiguous")
        n = param.numel()
        if phi.numel() != n * self.nn:
            raise ValueError("phi must hold %d x %d values" % (n, self.nn))
        return n, torch.cuda.current_stream(param.device).cuda_stream

    def chem_utils(self, phi, order="C", conp=True):
        """Species thermo at each state's (guarded) temperature: (cp, h, b), or
        (cv, u, b) when not conp; each (N, Ns) for order 'C', (Ns, N) for 'F'."""
        import torch
        if not (isinstance(phi, torch.Tensor) and phi.is_cuda and phi.dtype == torch.float64
                and phi.is_contiguous()):
            raise TypeError("expected a contiguous CUDA float64 tensor")
        if phi.numel() % self.nn:
            raise ValueError("phi must hold N x %d values" % self.nn)
        n = phi.numel() // self.nn
        ns = self.nn - 1
        shape = (n, ns) if order == "C" else (ns, n)
        out = [torch.empty(shape, dtype=torch.float64, device=phi.device) for _ in range(3)]
        st = torch.cuda.current_stream(phi.device).cuda_stream
        _lib.check("pjg_chem_utils", self._lib.pjg_chem_utils(
            self.handle, n, _order(order), int(bool(conp)), phi.data_ptr(), out[0].data_ptr(),
            out[1].data_ptr(), out[2].data_ptr(), st))
        return tuple(out)

    def species_rates(self, param, phi, order="C", conp=True, out=None):
        import torch
        n, st = self._prep(param, phi, order)
        if out is None:
            out = torch.empty_like(phi)
        _lib.check("pjg_species_rates", self._lib.pjg_species_rates(
            self.handle, n, _order(order), int(bool(conp)), param.data_ptr(), phi.data_ptr(),
            out.data_ptr(), st))
        return out

    def jacobian(self, param, phi, order="C", conp=True, jac_format="full", out=None, dphi=None):
        """The Jacobian; with ``dphi`` (a tensor like phi) the species rates of
        the same pass are written there too (pjg_jacobian_rates)."""
        import torch
        n, st = self._prep(param, phi, order)
        fmt = _fmt(jac_format)
        per = self.nn * self.nn if fmt == 0 else self.nnz
        if out is None:
            if order == "C":
                shape = (n, self.nn, self.nn) if fmt == 0 else (n, per)
            else:
                shape = (self.nn, self.nn, n) if fmt == 0 else (per, n)
            out = torch.empty(shape, dtype=torch.float64, device=phi.device)
        elif out.numel() != n * per:
            raise ValueError("output must hold %d values" % (n * per))
        if dphi is not None:
            if dphi.shape != phi.shape or dphi.dtype != torch.float64 or not dphi.is_contiguous():
                raise ValueError("dphi must match phi")
            _lib.check("pjg_jacobian_rates", self._lib.pjg_jacobian_rates(
                self.handle, n, _order(order), int(bool(conp)), fmt, param.data_ptr(),
                phi.data_ptr(), out.data_ptr(), dphi.data_ptr(), st))
            return out
        _lib.check("pjg_jacobian", self._lib.pjg_jacobian(
            self.handle, n, _order(order), int(bool(conp)), fmt, param.data_ptr(), phi.data_ptr(),
            out.data_ptr(), st))
        return out

    def vjp(self, param, phi, v, order="C", conp=True, out=None):
        import torch
        n, st = self._prep(param, phi, order)
        if v.shape != phi.shape or v.dtype != torch.float64 or not v.is_contiguous():
            raise ValueError("v must match phi")
        if out is None:
            out = torch.empty_like(phi)
        _lib.check("pjg_vjp", self._lib.pjg_vjp(
            self.handle, n, _order(order), int(bool(conp)), param.data_ptr(), phi.data_ptr(),
            v.data_ptr(), out.data_ptr(), st))
        return out


class _KernelBase(object):
    _kind = None

    def __init__(self, problem_size, work_size, do_not_compile=False, **kwargs):
        skip = kwargs.pop("testing_only_skip_compilation", False)
        if kwargs:
            raise TypeError("unexpected keyword arguments %s" % sorted(kwargs))
        self._dm = self._dev_mech()
        self._lib = self._dm._lib
        self.handle = ctypes.c_void_p()
        if not skip:
            self.resize(problem_size, work_size, do_not_compile)

    def resize(self, problem_size, work_size, do_not_compile=False):
        """Resize the device buffers (the reference's Kernel::resize)."""
        if not self.handle.value:
            h = ctypes.c_void_p()
            _lib.check("pjg_kernel_create", self._lib.pjg_kernel_create(
                self._dm.handle, self._kind, int(problem_size), int(work_size),
                self._order.encode(), int(self._conp), _fmt(self._jac_format), ctypes.byref(h)))
            self.handle = h
        else:
            _lib.check("pjg_kernel_resize", self._lib.pjg_kernel_resize(
                self.handle, int(problem_size), int(work_size)))
        self.problem_size = int(problem_size)
        self.work_size = int(work_size)

    def species_names(self):
        return self._mech.species_names()

    def reaction_strings(self):
        return self._mech.reaction_strings()

    def num_reactions(self):
        return self._mech.n_reactions

    def num_species(self):
        return self._mech.n_species

    def order(self):
        return self._order

    def required_working_memory(self):
        b = ctypes.c_size_t()
        _lib.check("pjg_kernel_required_memory",
                   self._lib.pjg_kernel_required_memory(self.handle, ctypes.byref(b)))
        return b.value

    def _out_size(self):
        n = self.problem_size
        if self._kind == KIND_RATES:
            return n * self._mech.nn
        if _fmt(self._jac_format) == 1:
            return n * self._dm.nnz
        return n * self._mech.nn * self._mech.nn

    def __call__(self, param, phi, out):
        n = self.problem_size
        arrs = [param, phi, out]
        sizes = [n, n * self._mech.nn, self._out_size()]
        for a, sz, name in zip(arrs, sizes, ("param", "phi", "output")):
            if not isinstance(a, np.ndarray) or a.dtype != np.float64:
                raise TypeError("%s must be a float64 numpy array" % name)
            if not (a.flags.c_contiguous or a.flags.f_contiguous) or a.size != sz:
                raise ValueError("%s must be a contiguous array of %d values" % (name, sz))
        if not out.flags.writeable:
            raise ValueError("output array is read-only")
        _lib.check("pjg_kernel_call", self._lib.pjg_kernel_call(
            self.handle, param.ctypes.data, phi.ctypes.data, out.ctypes.data))

    def close(self):
        if self.handle.value:
            self._lib.pjg_kernel_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pywrap(mech, order="C", conp=True, jac_format="full"):
    """Return a module-like namespace with PyJacobianKernel / PySpecies_RatesKernel.

    Equivalent to the ``pyjac_c`` module the reference generates for one
    mechanism and one set of options (pyjac/pywrap/pywrap_gen.py:249-345).
    """
    if order not in ("C", "F"):
        raise ValueError("order must be 'C' or 'F'")
    _fmt(jac_format)
    holder = {}

    def dev_mech():
        if "dm" not in holder:
            holder["dm"] = DeviceMechanism(mech)
        return holder["dm"]

    attrs = dict(_mech=mech, _order=order, _conp=bool(conp), _jac_format=jac_format,
                 _dev_mech=staticmethod(dev_mech))
    jk = type("PyJacobianKernel", (_KernelBase,), dict(attrs, _kind=KIND_JAC))
    rk = type("PySpecies_RatesKernel", (_KernelBase,), dict(attrs, _kind=KIND_RATES))
    ck = type("PyChem_UtilsKernel", (_ChemUtilsKernel,), attrs)
    return types.SimpleNamespace(PyJacobianKernel=jk, PySpecies_RatesKernel=rk,
                                 PyChem_UtilsKernel=ck, mechanism=mech, order=order,
                                 conp=bool(conp), jac_format=jac_format)


class _ChemUtilsKernel(object):
    """The chem_utils kernel type of the generated module: call(phi, cp, h, b)
    fills cp, h, b (cv, u, b when not conp), each Ns values per state in the
    kernel's order, from host arrays."""

    def __init__(self, problem_size, work_size, do_not_compile=False, **kwargs):
        kwargs.pop("testing_only_skip_compilation", None)
        if kwargs:
            raise TypeError("unexpected keyword arguments %s" % sorted(kwargs))
        self._ev = Evaluator(self._mech)
        self.resize(problem_size, work_size)

    def resize(self, problem_size, work_size, do_not_compile=False):
        self.problem_size = int(problem_size)
        self.work_size = int(work_size)

    def num_species(self):
        return self._mech.n_species

    def order(self):
        return self._order

    def __call__(self, phi, cp, h, b):
        import torch
        n, ns = self.problem_size, self._mech.n_species
        for a, sz, name in ((phi, n * (ns + 1), "phi"), (cp, n * ns, "cp"), (h, n * ns, "h"),
                            (b, n * ns, "b")):
            if not isinstance(a, np.ndarray) or a.dtype != np.float64 or a.size != sz:
                raise ValueError("%s must be a float64 numpy array of %d values" % (name, sz))
        x = torch.from_numpy(np.ascontiguousarray(phi).reshape(-1)).cuda()
        outs = self._ev.chem_utils(x, order=self._order, conp=self._conp)
        for host, dev in zip((cp, h, b), outs):
            host.reshape(-1)[:] = dev.reshape(-1).cpu().numpy()

    def close(self):
        pass
