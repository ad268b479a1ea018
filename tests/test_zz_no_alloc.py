"""The edge check without allocation (kgpu_check_edges_noalloc), called
through the C ABI: same first-hit indices as the regular entry point
(kgpu_check_edges) on two calls in a row with no device memory allocated by
either, the same results when its undecided-pair list overflows, and clear
errors past its fixed size limit and after the collision masks changed.  This file is collected last on purpose, so a failure here never
hides the results of the other tests; it also passes when run alone in a
fresh process."""

import ctypes
import os

import numpy as np
import pytest

from klampt_gb300 import scenes as sc

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_edges_match_regular_entry_point():
    import torch
    from klampt_gb300 import build, _kgpu
    from klampt_gb300.engine import World

    build.build()
    L = _kgpu.load()
    robot, env, (qa, qb, ns) = sc.scene_cfg1(n_edges=3000)
    w = World(env, [robot])
    a = torch.as_tensor(qa).cuda()
    b = torch.as_tensor(qb).cuda()
    n = torch.as_tensor(ns).cuda()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.empty(len(ns), dtype=torch.int32, device="cuda")
    _kgpu.check(L.kgpu_check_edges(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), len(ns), _dptr(ref), stream))
    _kgpu.check(L.kgpu_world_sync(w.handle, stream))
    ref_np = ref.cpu().numpy()
    assert (ref_np >= 0).any() and (ref_np < 0).any()
    from oracle.oracle_py import Oracle
    fo, _ = Oracle(robot, env).check_edges(qa, qb, ns, nthreads=os.cpu_count() or 4)
    bad = np.nonzero(ref_np != fo)[0]
    assert bad.size == 0, [(int(i), int(ref_np[i]), int(fo[i]), int(ns[i])) for i in bad[:8]]
    outs = [torch.full((len(ns),), -7, dtype=torch.int32, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for out in outs:  # two calls in a row share (and reuse) the static scratch
        _kgpu.check(L.kgpu_check_edges_noalloc(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), len(ns), _dptr(out),
                                               stream))
        _kgpu.check(L.kgpu_world_sync(w.handle, stream))
        out_np = out.cpu().numpy()
        bad = np.nonzero(out_np != ref_np)[0]
        assert bad.size == 0, [(int(i), int(out_np[i]), int(ref_np[i]), int(ns[i])) for i in bad[:8]]
    # nothing was allocated on the device by either call (the array was
    # loaded when the world was created)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    # the undecided-pair list capped at one entry: the fallback pass re-checks
    # every step with the FP64 test inline, and the results stay the same
    w.set_option("pend_cap", 1)
    out = outs[0]
    out.fill_(-7)
    _kgpu.check(L.kgpu_check_edges_noalloc(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), len(ns), _dptr(out), stream))
    _kgpu.check(L.kgpu_world_sync(w.handle, stream))
    assert np.array_equal(out.cpu().numpy(), ref_np)
    w.set_option("pend_cap", 0)
    # beyond the fixed maximum: rejected with a message, nothing launched
    st = L.kgpu_check_edges_noalloc(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), 65537, _dptr(out), stream)
    assert st == _kgpu.KGPU_ERR_INVALID
    assert "65536" in _kgpu.last_error()
    # collision masks changed since the last regular query: re-uploading them
    # would allocate, so the call is rejected until a regular query ran
    w.enable_self_pair(0, 0, 6, False)
    st = L.kgpu_check_edges_noalloc(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), len(ns), _dptr(out), stream)
    assert st == _kgpu.KGPU_ERR_INVALID
    assert "masks" in _kgpu.last_error()
    w.check_edges(a, b, n)
    _kgpu.check(L.kgpu_check_edges_noalloc(w.handle, 0, _dptr(a), _dptr(b), _dptr(n), len(ns), _dptr(out), stream))
    _kgpu.check(L.kgpu_world_sync(w.handle, stream))
    w.close()
