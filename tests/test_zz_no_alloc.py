"""The allocation-free body-force entry point, lbm_body_force_f32_noalloc.

Callers that cannot allocate device memory (a host framework that has
reserved the device's memory for its own pool, a real-time loop that cannot
afford cudaMalloc, a plugin host that forbids allocation) use this variant of
lbm_body_force_f32: it keeps its partial sums in a fixed array of the
library's device memory instead of a caller-provided scratch buffer.  This
test calls it through the C ABI twice in a row, on two different population
states, and checks each result against the scratch-buffer entry point, then
against the handle's own drag/lift and its accumulation into force_out.  The
file is named to be collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX, NY, NZ, PITCH = 64, 24, 6, 64


def test_noalloc_force_matches_scratch_version_twice(product):
    torch = pytest.importorskip("torch")
    lbm = product
    lib = lbm.library()
    text = lbm.make_inputs(NX, NY, NZ, obst1=(20.5, 11.5, 0.0), r1=4.0, re=60.0, umax=0.05, tmax=20, les=1,
                           cs=0.01, geometry="channel_square")
    states = []
    with lbm.Solver(text) as s:
        mask = s.mask()
        s.step(3)
        states.append(s.populations())
        s.step(5)
        states.append(s.populations())
    assert (mask == lbm.NODE["BODY"]).any()
    dev = torch.device("cuda", torch.cuda.current_device())
    m = torch.full((NZ, NY, PITCH), lbm.NODE["WALL"], dtype=torch.uint8, device=dev)
    m[..., :NX] = torch.from_numpy(mask).to(dev)
    scratch = torch.zeros(int(lib.lbm_body_force_scratch_doubles()), dtype=torch.float64, device=dev)
    P = ctypes.c_void_p
    stream = P(torch.cuda.current_stream().cuda_stream)
    for f in states:
        fa = torch.zeros((19, NZ, NY, PITCH), dtype=torch.float32, device=dev)
        fa[..., :NX] = torch.from_numpy(f).to(dev)
        want = torch.zeros(3, dtype=torch.float64, device=dev)
        got = torch.zeros(3, dtype=torch.float64, device=dev)
        assert lib.lbm_body_force_f32(P(fa.data_ptr()), P(m.data_ptr()), NX, NY, NZ, PITCH, P(want.data_ptr()),
                                      P(scratch.data_ptr()), stream) == 0, lib.lbm_last_error()
        assert lib.lbm_body_force_f32_noalloc(P(fa.data_ptr()), P(m.data_ptr()), NX, NY, NZ, PITCH,
                                              P(got.data_ptr()), stream) == 0, lib.lbm_last_error()
        torch.cuda.synchronize()
        w, g = want.cpu().numpy(), got.cpu().numpy()
        assert np.abs(w[0]) > 0.1
        np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-12)


def test_noalloc_force_matches_handle_and_accumulates(product):
    """the allocation-free reduction against the handle's own drag/lift of
    the same populations (its force history entry for the next step), and
    its documented accumulation: two calls on a non-default stream into a
    force_out that starts non-zero add twice the force"""
    torch = pytest.importorskip("torch")
    lbm = product
    lib = lbm.library()
    text = lbm.make_inputs(NX, NY, NZ, obst1=(20.5, 11.5, 0.0), r1=4.0, re=60.0, umax=0.05, tmax=20, les=1,
                           cs=0.01, geometry="channel_square")
    k = 6
    with lbm.Solver(text) as s:
        mask = s.mask()
        s.step(k)
        f = s.populations()
        s.step(1)
        F_handle = s.forces()[k]
    dev = torch.device("cuda", torch.cuda.current_device())
    m = torch.full((NZ, NY, PITCH), lbm.NODE["WALL"], dtype=torch.uint8, device=dev)
    m[..., :NX] = torch.from_numpy(mask).to(dev)
    fa = torch.zeros((19, NZ, NY, PITCH), dtype=torch.float32, device=dev)
    fa[..., :NX] = torch.from_numpy(f).to(dev)
    start = torch.tensor([1.5, -2.0, 0.25], dtype=torch.float64, device=dev)
    got = start.clone()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    P = ctypes.c_void_p
    for _ in range(2):
        assert lib.lbm_body_force_f32_noalloc(P(fa.data_ptr()), P(m.data_ptr()), NX, NY, NZ, PITCH,
                                              P(got.data_ptr()), P(side.cuda_stream)) == 0, lib.lbm_last_error()
    side.synchronize()
    once = (got - start).cpu().numpy() / 2
    assert abs(F_handle[0]) > 0.1
    np.testing.assert_allclose(once, F_handle, rtol=1e-12, atol=1e-12)


def test_noalloc_rejects_oversized_domains(product):
    lib = product.library()
    P = ctypes.c_void_p
    # 19 * 2048 * 2048 * 2048 elements cannot be indexed in 32 bits: rejected before any launch
    rc = lib.lbm_body_force_f32_noalloc(P(16), P(16), 2048, 2048, 2048, 2048, P(16), None)
    assert rc == 1 and b"2^31" in lib.lbm_last_error()
