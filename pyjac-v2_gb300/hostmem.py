"""Pinned host arrays for the kernel objects' host-pointer calls.

``empty(shape)`` maps anonymous memory, asks for transparent huge pages
(``madvise``, best effort), touches every page from the CPU, and page-locks
the range in place with ``pjg_host_register`` (cudaHostRegister).  The array
keeps the mapping and the registration alive; both are released when the
array is garbage-collected (keep the array itself alive while views of it are
in use).  On GB300, after other processes had churned host
memory, dense Jacobian calls into such buffers took 145-210 ms per 1M GRI
states, against 146-334 ms (alternating) into cudaHostAlloc'd ones.
"""
import ctypes
import mmap
import weakref

import numpy as np

from . import _lib

_MADV_HUGEPAGE = 14
_keep = {}


def _release(key):
    m = _keep.pop(key, None)
    if m is None:
        return
    mem, addr = m
    try:
        _lib.load().pjg_host_unregister(ctypes.c_void_p(addr))
        mem.close()
    except (BufferError, RuntimeError, ValueError):
        pass  # at interpreter exit views may still exist; the OS reclaims the mapping


def empty(shape, dtype=np.float64):
    """A page-locked numpy array (uninitialised apart from the touch)."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    if nbytes == 0:
        return np.empty(shape, dtype=dtype)
    mem = mmap.mmap(-1, nbytes, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
    raw = np.frombuffer(mem, dtype=np.uint8)
    addr = raw.ctypes.data
    try:
        libc = ctypes.CDLL(None, use_errno=True)
        libc.madvise(ctypes.c_void_p(addr), ctypes.c_size_t(nbytes), _MADV_HUGEPAGE)
    except (OSError, AttributeError):
        pass
    raw[::mmap.PAGESIZE] = 0  # fault every page in from the CPU
    rc = _lib.load().pjg_host_register(ctypes.c_void_p(addr), nbytes)
    if rc != 0:
        del raw
        mem.close()
        _lib.check("pjg_host_register", rc)
    arr = raw.view(dtype).reshape(shape)
    key = id(mem)
    _keep[key] = (mem, addr)
    weakref.finalize(arr, _release, key)
    del raw
    return arr
