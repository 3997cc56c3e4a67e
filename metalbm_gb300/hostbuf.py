"""Page-locked host arrays for the C ABI's host<->device copies.

`pinned_array(shape)` maps anonymous memory aligned to the kernel's
transparent-huge-page size (hpage_pmd_size: 2 MiB with 4 KiB base pages,
512 MiB with the 64 KiB base pages of GB300 hosts), asks for transparent huge
pages (madvise MADV_HUGEPAGE) and registers the range with CUDA
(cudaHostRegister). Without the alignment a mapping gets few or no huge pages
of that size. On GB300 hosts with 64 KiB pages the transfers of the 4.3 GB
field arrays of a 512^3 lattice were bound by the translation of the host
pages: the copy engines uploaded them in 300-450 ms, a copy kernel over the
host link in ~30 ms with warm translations and ~300 ms with cold ones (those
hosts granted no 512 MiB transparent huge page, aligned or not).
"""
from __future__ import annotations

import mmap
import weakref

import numpy as np


def _cudart():
    import torch
    return torch.cuda.cudart()


def _thp_size() -> int:
    """The transparent-huge-page (PMD) size of this kernel, 2 MiB if unknown."""
    try:
        with open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size") as fh:
            n = int(fh.read().strip())
        return n if n > 0 and n & (n - 1) == 0 else 1 << 21
    except (OSError, ValueError):
        return 1 << 21


def pinned_array(shape, dtype=np.float64) -> np.ndarray:
    """Zero-filled, page-locked numpy array, aligned to the huge-page size and
    backed by huge pages when the kernel grants them; unregistered and
    unmapped when garbage-collected."""
    dtype = np.dtype(dtype)
    count = int(np.prod(shape))
    nbytes = max(count * dtype.itemsize, 1)
    huge = _thp_size()
    # large arrays: a mapping one huge page longer, the array at its first
    # huge-page boundary
    align = huge if nbytes >= huge else mmap.PAGESIZE
    mm = mmap.mmap(-1, nbytes + align, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
    base = np.frombuffer(mm, dtype=np.uint8)
    addr = base.ctypes.data
    offset = (-addr) % align
    if hasattr(mmap, "MADV_HUGEPAGE"):
        try:
            mm.madvise(mmap.MADV_HUGEPAGE)
        except OSError:
            pass  # huge pages are an optimisation; the registration below still pins
    arr = base[offset:offset + count * dtype.itemsize].view(dtype).reshape(shape)
    arr[...] = 0  # fault every page in before registration
    rt = _cudart()
    rc = rt.cudaHostRegister(arr.ctypes.data, nbytes, 0)
    code = rc[0] if isinstance(rc, tuple) else rc
    if int(code) != 0:
        raise RuntimeError(f"cudaHostRegister failed ({int(code)})")
    ptr = arr.ctypes.data

    def _release(ptr=ptr, mm=mm):
        try:
            _cudart().cudaHostUnregister(ptr)
        except Exception:
            pass
        # the mapping closes with the last reference to `mm`

    weakref.finalize(arr, _release)
    return arr
