"""The broken-bond listing that allocates nothing, against the backend's own answers.

gbl_broken_between_noalloc serves callers that may not allocate device memory
while they run (a real-time frame loop, or work being recorded into a CUDA
graph): it lists the bonds that broke between two aliveness snapshots with its
scratch in a fixed static device array. Here its lists must equal what the
backend reports through its existing entry points -- the first failure round
from gbl_first_failure_bonds, a later window from two gbl_download snapshots --
on two calls in a row that share the array. This file is collected last so a
stop-at-first-failure run has already run every other test; it also passes
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    for path in ("/usr/local/cuda/lib64/libcudart.so", "/usr/local/cuda/targets/sbsa-linux/lib/libcudart.so",
                 "/usr/local/cuda/targets/x86_64-linux/lib/libcudart.so", "libcudart.so"):
        try:
            return ctypes.CDLL(path)
        except OSError:
            continue
    pytest.fail("libcudart not found")


class DeviceBuffer:
    """Test-side device memory (the entry point under test allocates none)."""

    def __init__(self, rt, nbytes):
        self.rt = rt
        self.ptr = ctypes.c_void_p()
        assert rt.cudaMalloc(ctypes.byref(self.ptr), ctypes.c_size_t(max(nbytes, 4))) == 0
        self.nbytes = nbytes

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        assert self.rt.cudaMemcpy(self.ptr, arr.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(arr.nbytes), 1) == 0

    def get(self, dtype, count):
        out = np.empty(count, dtype=dtype)
        if count:
            assert self.rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), self.ptr, ctypes.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.ptr)


def _list_broken(lib, rt, before, after, d_before, d_after, d_out, d_count):
    d_before.put(before)
    d_after.put(after)
    lib.gbl_broken_between_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]
    rc = lib.gbl_broken_between_noalloc(d_before.ptr, d_after.ptr, before.size, d_out.ptr, d_count.ptr, None)
    assert rc == 0
    assert rt.cudaDeviceSynchronize() == 0
    n = int(d_count.get(np.uint32, 1)[0])
    return d_out.get(np.uint32, n)


def test_noalloc_listing_matches_backend_twice_in_a_row(device):
    from banjo_gb300 import scenes

    lib = device.library()
    rt = _cudart()
    case = scenes.cantilever(steps=4)  # first failure at substep 19
    n = int(case["node_count"][0])
    sched = device.build_lattice_schedule(n, case["bond_a"], case["bond_b"], case["node_block_begin"])
    state = device.build_lattice_state(case, sched)
    be = device.make_gb300_lattice_backend(sched)
    be.upload(state, device.step_settings(case["settings"]), device.sphere_state(case["sphere"]))
    be.set_external_forces(case["forces"], int(case["force_substeps"][0]))
    st = be.run(device.RunControl(max_steps=19))
    assert st.broken_bonds == 0
    be.download(state)
    alive_19 = state.alive.copy()
    st = be.run(device.RunControl(max_steps=1))
    assert st.first_failure_step == 19 and st.broken_bonds > 0
    be.download(state)
    alive_20 = state.alive.copy()
    first = be.first_failure_bonds()
    be.run(device.RunControl(max_steps=15))
    be.download(state)
    alive_35 = state.alive.copy()
    later = np.nonzero((alive_20 != 0) & (alive_35 == 0))[0].astype(np.uint32)
    assert later.size > first.size > 0

    B = alive_19.size
    bufs = [DeviceBuffer(rt, B), DeviceBuffer(rt, B), DeviceBuffer(rt, 4 * B), DeviceBuffer(rt, 4)]
    try:
        got_first = _list_broken(lib, rt, alive_19, alive_20, *bufs)
        got_later = _list_broken(lib, rt, alive_20, alive_35, *bufs)
        assert np.array_equal(got_first, first)
        assert np.array_equal(got_later, later)
        # A third call over the same snapshots as the first: the shared scratch
        # holds the second call's tiles and must not leak into the answer.
        assert np.array_equal(_list_broken(lib, rt, alive_19, alive_20, *bufs), first)
    finally:
        for b in bufs:
            b.free()


def test_noalloc_listing_refuses_sizes_beyond_its_scratch(device):
    lib = device.library()
    lib.gbl_broken_between_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]
    rc = lib.gbl_broken_between_noalloc(None, None, (1 << 27) + 1, None, None, None)
    assert rc == 1
    buf = ctypes.create_string_buffer(256)
    lib.gbl_last_error(buf, 256)
    assert b"134217728" in buf.value


@pytest.mark.parametrize("bond_count,seed", [(10_000_019, 3), ((1 << 27) - 5, 4), (1 << 27, 5)])
def test_noalloc_listing_over_many_tiles(device, bond_count, seed):
    """Random snapshots of more than 1024 tiles of 8192 bonds: every scan
    thread adds up several tiles, and the list crosses every tile and warp
    boundary of the emission. The expected list is numpy's."""
    lib = device.library()
    rt = _cudart()
    rng = np.random.default_rng(seed)
    before = (rng.random(bond_count) < 0.9).astype(np.uint8)
    after = before & (rng.random(bond_count) < 0.97).astype(np.uint8)
    # A few runs of breaks that cross tile boundaries, and a broken last bond.
    for edge in (8192, 8192 * 1024, 8192 * 1200):
        if edge + 40 < bond_count:
            before[edge - 40:edge + 40] = 1
            after[edge - 40:edge + 40] = 0
    before[-1], after[-1] = 1, 0
    expected = np.nonzero((before != 0) & (after == 0))[0].astype(np.uint32)
    # The output has room for every bond, as the entry point asks.
    bufs = [DeviceBuffer(rt, bond_count), DeviceBuffer(rt, bond_count), DeviceBuffer(rt, 4 * bond_count),
            DeviceBuffer(rt, 4)]
    try:
        got = _list_broken(lib, rt, before, after, *bufs)
        assert got.size == expected.size
        assert np.array_equal(got, expected)
    finally:
        for b in bufs:
            b.free()
