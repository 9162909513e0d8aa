"""sqdem_contacts_static_queue: the contact stage for callers that cannot allocate device
memory at the point where they advance contacts (a host framework that owns device memory
through its own pool and forbids raw cudaMalloc after start-up, or a loop that must not block
in the allocator).  Its work queue lives in a fixed static device array instead of a buffer
the context allocated; the results must equal those of the allocating path
(sqdem_time_contacts) on the same state, call after call, also when the call is queued
straight behind unsynchronised timesteps.

This file is collected last on purpose, so a failure here does not stop the other tests.
"""
import numpy as np
import pytest

from sudodem_gb300 import Engine, SqdemError, assemblies

pytestmark = pytest.mark.gpu


def _pair_of_engines(spec, warm_steps=3):
    a, b = Engine(device=0), Engine(device=0)
    a.load(spec)
    b.load(spec)
    a.step(warm_steps)
    b.step(warm_steps)
    a.sync()
    b.sync()
    assert np.array_equal(a.interactions(True), b.interactions(True))
    return a, b


def test_static_queue_matches_allocating_path_twice(gpu):
    spec = assemblies.walled_lattice(400, seed=5, box=14e-3, per_side=5, spacing=2.1e-3)
    ref, noalloc = _pair_of_engines(spec)
    for _ in range(2):
        ref.time_contacts(1)               # existing entry point, context-owned queue
        noalloc.contacts_static_queue()    # static-array queue, no allocation
        ref.sync()
        noalloc.sync()
        ri, ni = ref.interactions(True), noalloc.interactions(True)
        assert ri.shape == ni.shape and len(ri) > 1000
        # same tolerance as the GPU parity tests for identical inputs: bit for bit
        assert np.array_equal(ri, ni)
        touching = np.sum(ni[:, 4] > 0)
        assert touching > 50


def test_static_queue_after_unsynchronised_steps_allocates_nothing(gpu):
    """Queued directly behind asynchronous timesteps (no sync between), the call must see
    their table, and a second call must leave the device's free memory unchanged."""
    import torch
    spec = assemblies.walled_lattice(400, seed=7, box=14e-3, per_side=5, spacing=2.1e-3)
    ref, noalloc = Engine(device=0), Engine(device=0)
    ref.load(spec)
    noalloc.load(spec)
    ref.step(4)
    ref.time_contacts(1)
    noalloc.step(4)
    noalloc.contacts_static_queue()        # no sync after step(): ordered on the stream
    ref.sync()
    noalloc.sync()
    assert np.array_equal(ref.interactions(True), noalloc.interactions(True))
    free_before = torch.cuda.mem_get_info(0)[0]
    noalloc.contacts_static_queue()
    noalloc.sync()
    free_after = torch.cuda.mem_get_info(0)[0]
    assert free_after == free_before
    ref.time_contacts(1)
    ref.sync()
    assert np.array_equal(ref.interactions(True), noalloc.interactions(True))


def test_static_queue_rejects_tables_beyond_its_size(gpu):
    spec = assemblies.deposition_box(150_000, seed=1)
    e = Engine(device=0)
    e.load(spec)
    e.step(1)
    e.sync()
    n = len(e.interactions(True))
    assert n > (1 << 20)
    with pytest.raises(SqdemError) as ei:
        e.contacts_static_queue()
    assert ei.value.status == 3
    # a context of the same scene with a table small enough for the array is accepted
    small = assemblies.walled_lattice(400, seed=5, box=14e-3, per_side=5, spacing=2.1e-3)
    ok = Engine(device=0, contacts_per_body=16)
    ok.load(small)
    ok.contacts_static_queue()
    ok.sync()
