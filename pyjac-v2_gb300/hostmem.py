"""Pinned host arrays for the kernel objects' host-pointer calls.

``empty(shape)`` maps anonymous memory, asks for transparent huge pages
(``madvise``, best effort), optionally binds it to one NUMA node
(``mbind``; ``node="gpu"`` picks the node the GPU's PCI device reports),
touches every page from the CPU, and page-locks the range in place with
``pjg_host_register`` (cudaHostRegister).  ``placement_info`` reports on
which NUMA nodes an array's pages landed.  The array
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
_MPOL_BIND = 2
_SYS_MBIND = {"aarch64": 235, "x86_64": 237}
_keep = {}


def gpu_numa_node(device=0):
    """The NUMA node of the GPU's PCI device (its nearest host memory), or None."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(device)
        bdf = "%04x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        with open("/sys/bus/pci/devices/%s/numa_node" % bdf) as fh:
            node = int(fh.read().strip())
        return node if node >= 0 else None
    except (AttributeError, OSError, ValueError, RuntimeError, ImportError):
        return None


def _mbind(addr, nbytes, node):
    """Bind [addr, addr + nbytes) to NUMA node `node` before its pages are
    touched; False where the system call is unavailable or refused."""
    import platform
    nr = _SYS_MBIND.get(platform.machine())
    if nr is None or node is None or not 0 <= node < 64:
        return False
    try:
        libc = ctypes.CDLL(None, use_errno=True)
        mask = ctypes.c_ulong(1 << node)
        rc = libc.syscall(ctypes.c_long(nr), ctypes.c_void_p(addr), ctypes.c_ulong(nbytes),
                          ctypes.c_int(_MPOL_BIND), ctypes.byref(mask), ctypes.c_ulong(65),
                          ctypes.c_uint(0))
        return rc == 0
    except (OSError, AttributeError):
        return False


def placement_info(arr):
    """{'host_numa_pages': {node: pages}, 'gpu_numa_node': n} for the pages of
    `arr` (from /proc/self/numa_maps); empty where that file is unavailable."""
    lo = arr.ctypes.data
    hi = lo + arr.nbytes
    pages = {}
    try:
        with open("/proc/self/numa_maps") as fh:
            for line in fh:
                parts = line.split()
                start = int(parts[0], 16)
                if not lo <= start < hi:
                    continue
                for p in parts[1:]:
                    if p.startswith("N") and "=" in p:
                        k, v = p.split("=", 1)
                        pages[k] = pages.get(k, 0) + int(v)
    except (OSError, ValueError, IndexError):
        return {}
    return {"host_numa_pages": pages, "gpu_numa_node": gpu_numa_node()}


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


def empty(shape, dtype=np.float64, node=None):
    """A page-locked numpy array (uninitialised apart from the touch).
    node: None (the first-touch policy of the calling thread), a NUMA node
    number, or "gpu" (the GPU's node, gpu_numa_node())."""
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
    if node is not None:
        _mbind(addr, nbytes, gpu_numa_node() if node == "gpu" else int(node))
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
