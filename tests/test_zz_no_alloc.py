"""rsg_air_backward_noalloc (the air adjoint with its tape in a static device array) against
rsg_air_backward with a caller workspace, through the C ABI, on two calls in a row."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from air_cases import gradient_case

pytestmark = pytest.mark.gpu


def test_noalloc_backward_matches_workspace_backward():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rocketsim_gb300 as rsg
    from rocketsim_gb300 import abi
    lib = abi.load(build_if_missing=False)
    cfg = rsg.car_config(abi.CAR_OCTANE)
    P = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    n, ticks, every = 1500, 60, 16  # 90000 instance-ticks, inside the 110376 limit
    for call, seed in enumerate((21, 22)):  # two calls in a row, different inputs
        s, u, _ = gradient_case(seed, n, ticks)
        ds = torch.from_numpy(s).cuda()
        du = torch.from_numpy(u).cuda()
        fin = torch.empty_like(ds)
        ck = torch.empty(((ticks + every - 1) // every, n, 24), device="cuda")
        abi.check(lib.rsg_air_forward(C.byref(cfg), 120.0, n, ticks, P(ds), P(du), P(fin), P(ck), every, None),
                  "rsg_air_forward")
        gfin = torch.from_numpy(np.random.default_rng(seed).normal(size=(n, 24)).astype(np.float32)).cuda()
        nb = C.c_size_t()
        abi.check(lib.rsg_air_backward_workspace_size(n, ticks, C.byref(nb)), "workspace size")
        work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
        gu_ref, gs_ref = torch.empty_like(du), torch.empty_like(ds)
        abi.check(lib.rsg_air_backward(C.byref(cfg), 120.0, n, ticks, P(du), P(ck), every, P(gfin), P(gu_ref),
                                       P(gs_ref), P(work), nb.value, None), "rsg_air_backward")
        gu, gs = torch.full_like(du, float("nan")), torch.full_like(ds, float("nan"))
        abi.check(lib.rsg_air_backward_noalloc(C.byref(cfg), 120.0, n, ticks, P(du), P(ck), every, P(gfin), P(gu),
                                               P(gs), None), "rsg_air_backward_noalloc")
        torch.cuda.synchronize()
        for got, ref in ((gu, gu_ref), (gs, gs_ref)):
            assert torch.isfinite(got).all(), call
            rel = ((got - ref).norm() / ref.norm()).item()
            assert rel <= 1e-6, (call, rel)
    # above the static array's size: a clear error and nothing launched
    big = 110377
    rc = lib.rsg_air_backward_noalloc(C.byref(cfg), 120.0, big, 1, P(du), P(ck), every, P(gfin), P(gu), None, None)
    assert rc == abi.ERR_ARG
    assert "static scratch" in abi.last_error()
