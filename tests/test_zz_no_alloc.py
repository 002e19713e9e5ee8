"""emoo_sort_permutation_noalloc: the sort permutation for callers that
cannot allocate device memory (a host whose pool allocator owns all device
memory, or a loop that must not take the synchronisation cudaMalloc can
cause). All of its scratch is a fixed array inside the library.

Checked through the C ABI against the existing entry point: the permutation
emoo_sort applies to a handle's particles (read back through their ids) must
equal the one the allocation-free call returns for the same keys, exactly,
on two different inputs in a row (the second call reuses the array the first
one left behind). This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from apc_524_project_gb300 import abi, configs, loading
from backends import GpuBackend

pytestmark = pytest.mark.gpu


def _case(n_cells, ppc, seed, nspecies_test=False):
    cfg = configs.tiny("noalloc", n=n_cells, ppc=ppc, init="constant", seed=seed, test_species=nspecies_test)
    info = configs.input_info(cfg)
    parts = loading.sample_all(cfg)
    g = GpuBackend(info, 0.4)
    nid = 0
    for si, p in enumerate(parts):
        g.add_species(si, p, ids=np.arange(nid, nid + len(p["x"])))
        nid += len(p["x"])
    # keys as emoo_sort builds them: species * ncell + reference cellID
    ncell = (cfg.n[0] + 2) * (cfg.n[1] + 2) * (cfg.n[2] + 2)
    keys = []
    for si, p in enumerate(parts):
        for x, y, z in zip(p["x"], p["y"], p["z"]):
            keys.append(si * ncell + g.cell_id(x, y, z))
    keys = np.array(keys, dtype=np.uint32)
    bits = int(len(parts) * ncell + 2).bit_length()
    g.sort()
    expected = g.particles()["id"].astype(np.uint32)
    g.close()
    return keys, bits, expected


def _noalloc(keys, bits):
    import torch

    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dp = torch.empty(len(keys), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = abi.lib().emoo_sort_permutation_noalloc(C.c_void_p(dk.data_ptr()), len(keys), bits,
                                                 C.c_void_p(dp.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, dp.cpu().numpy().view(np.uint32)


def test_noalloc_permutation_matches_emoo_sort_twice():
    k1, b1, e1 = _case((9, 8, 7), 6, 11, nspecies_test=True)
    k2, b2, e2 = _case((12, 5, 9), 5, 29)
    rc, p1 = _noalloc(k1, b1)
    assert rc == abi.OK
    np.testing.assert_array_equal(p1, e1)
    rc, p2 = _noalloc(k2, b2)
    assert rc == abi.OK
    np.testing.assert_array_equal(p2, e2)
    # the permutation sorts the keys, equal keys in input order
    s = k2[p2]
    assert np.all(np.diff(s.astype(np.int64)) >= 0)


def test_noalloc_rejects_sizes_beyond_its_array():
    import torch

    d = torch.empty(4, dtype=torch.int32, device="cuda")
    ptr = C.c_void_p(d.data_ptr())
    L = abi.lib()
    assert L.emoo_sort_permutation_noalloc(ptr, abi.NOALLOC_SORT_MAX + 1, 16, ptr, None) == abi.ERR_ARG
    assert L.emoo_sort_permutation_noalloc(ptr, -1, 16, ptr, None) == abi.ERR_ARG
    assert L.emoo_sort_permutation_noalloc(ptr, 4, 33, ptr, None) == abi.ERR_ARG
    assert L.emoo_sort_permutation_noalloc(ptr, 0, 16, ptr, None) == abi.OK
