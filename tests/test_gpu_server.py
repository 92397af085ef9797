"""GPU tests of the culling server: results against the oracle, the same
bits alone and in a concurrent mix, copy-on-write light updates and device
jitter (checked against its host restatement), budget admission and
eviction, and a short run of the Poisson load driver."""
import numpy as np
import pytest

from hellovulkan_gb300 import scenes

pytestmark = pytest.mark.gpu


def oracle_result(oracle, ubo, lights, cap=150):
    a = oracle.generate_aabbs(ubo)
    cells, idx, _ = oracle.cull(ubo, a, lights, cap)
    return cells, idx


def take(srv, count):
    out = srv.wait_all(count)
    assert len(out) == count
    return {c.request_id: c for c in out}


def test_server_results_match_the_oracle(gpu, oracle):
    from hellovulkan_gb300.server import Server
    srv = Server(gpu, budget_bytes=1 << 30)
    rng = np.random.default_rng(1)
    views = [scenes.batch_view(rng) for _ in range(6)]
    reqs = {}
    for v in views:
        lights = v.lights[:4000]
        sid = srv.register(lights)
        reqs[srv.submit(v.ubo, sid)] = (v.ubo, lights)
    for rid, c in take(srv, len(reqs)).items():
        assert c.status == 0
        cells, idx = srv.read(c)
        oc, oi = oracle_result(oracle, *reqs[rid])
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi)
        srv.release(rid)
    st = srv.stats()
    assert st["completed"] == len(views) and st["resident_projections"] >= 1
    srv.close()


def test_same_result_alone_and_in_a_concurrent_mix(gpu, oracle):
    from hellovulkan_gb300.server import Server
    srv = Server(gpu, budget_bytes=2 << 30, max_batch_views=16, streams=4)
    rng = np.random.default_rng(2)
    probe = scenes.batch_view(rng)
    probe_lights = probe.lights[:5000]
    sid = srv.register(probe_lights)
    # alone
    rid = srv.submit(probe.ubo, sid)
    c = take(srv, 1)[rid]
    alone = srv.read(c)
    srv.release(rid)
    # in a mix: 120 other requests around it, over several batches and streams
    others = []
    for k in range(60):
        v = scenes.batch_view(rng)
        others.append((v.ubo, srv.register(v.lights[:3000])))
    ids = [srv.submit(u, s) for u, s in others[:40]]
    rid2 = srv.submit(probe.ubo, sid)
    ids += [srv.submit(u, s) for u, s in others[40:]] + [srv.submit(u, s) for u, s in others]
    done = take(srv, len(ids) + 1)
    mixed = srv.read(done[rid2])
    for r in done:
        srv.release(r)
    assert np.array_equal(alone[0], mixed[0]) and np.array_equal(alone[1], mixed[1])
    oc, oi = oracle_result(oracle, probe.ubo, probe_lights)
    assert np.array_equal(mixed[0], oc) and np.array_equal(mixed[1], oi)
    assert srv.stats()["batches"] >= 2
    srv.close()


def test_copy_on_write_updates_and_device_jitter(gpu, oracle):
    from hellovulkan_gb300.server import Server
    from oracle import jitter_lights
    srv = Server(gpu, budget_bytes=1 << 30)
    v = scenes.plain_small(3)
    sid = srv.register(v.lights)
    r1 = srv.submit(v.ubo, sid)
    moved = v.lights.copy()
    moved[:, :3] += 0.75
    srv.update(sid, moved)  # r1 keeps the version it was submitted with
    r2 = srv.submit(v.ubo, sid)
    srv.jitter(sid, 1234, 0.1)
    r3 = srv.submit(v.ubo, sid)
    done = take(srv, 3)
    res = {r: srv.read(done[r]) for r in (r1, r2, r3)}
    for r in done:
        srv.release(r)
    oc, oi = oracle_result(oracle, v.ubo, v.lights)
    assert np.array_equal(res[r1][0], oc) and np.array_equal(res[r1][1], oi)
    oc, oi = oracle_result(oracle, v.ubo, moved)
    assert np.array_equal(res[r2][0], oc) and np.array_equal(res[r2][1], oi)
    jittered = jitter_lights(moved, 1234, 0.1)
    assert not np.array_equal(jittered, moved)
    oc, oi = oracle_result(oracle, v.ubo, jittered)
    assert np.array_equal(res[r3][0], oc) and np.array_equal(res[r3][1], oi)
    srv.close()


def test_release_many_returns_every_output_and_reports_unknown_ids(gpu):
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.server import Server
    srv = Server(gpu, budget_bytes=256 << 20)
    v = scenes.plain_small(6)
    sid = srv.register(v.lights)
    ids = [srv.submit(v.ubo, sid) for _ in range(12)]
    take(srv, len(ids))
    held = srv.stats()["arena_used_bytes"]
    with pytest.raises(CfError) as e:
        srv.release_many(ids + [10 ** 9])  # one id that holds nothing: the others are still released
    assert e.value.status == 1  # CF_ERROR_INVALID_ARGUMENT
    assert srv.stats()["arena_used_bytes"] < held
    with pytest.raises(CfError):
        srv.release(ids[0])  # already released
    srv.release_many([])
    assert srv.stats()["max_held_outputs"] == 12
    srv.close()


def test_declared_pinned_ranges(gpu, oracle):
    """Registers and updates from inside a declared pinned range make no CUDA
    call and give the oracle's result; undeclared pinned memory still works;
    pageable and overlapping declarations are refused."""
    torch = pytest.importorskip("torch")
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.server import Server
    srv = Server(gpu, budget_bytes=256 << 20)
    rng = np.random.default_rng(8)
    v = scenes.plain_small(7)
    pool = torch.from_numpy(np.ascontiguousarray(
        scenes.uniform_box_lights(rng, 3000, [-20, -10, -60], [20, 10, -1], 1.0, 6.0), np.float32)).pin_memory()
    srv.declare_pinned(pool)
    srv.declare_pinned(pool)  # the same range again: a no-op
    with pytest.raises(CfError) as e:
        srv.declare_pinned(pool[1000:2000])  # inside a declared range
    assert e.value.status == 1
    with pytest.raises(CfError) as e:
        srv.declare_pinned(np.zeros((100, 12), np.float32))  # pageable
    assert e.value.status == 1
    a = pool.numpy()
    expect = {}
    s1 = srv.register(a[100:1100])  # 100 lights in: still 16-byte aligned
    expect[srv.submit(v.ubo, s1)] = a[100:1100].copy()
    srv.update(s1, a[2000:2900])
    expect[srv.submit(v.ubo, s1)] = a[2000:2900].copy()
    other = torch.from_numpy(np.ascontiguousarray(a[:700])).pin_memory()  # pinned, undeclared
    s2 = srv.register(other.numpy())
    expect[srv.submit(v.ubo, s2)] = a[:700].copy()
    done = take(srv, len(expect))
    for rid, lights in expect.items():
        cells, idx = srv.read(done[rid])
        oc, oi = oracle_result(oracle, v.ubo, lights)
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi), rid
    srv.release_many(list(expect))
    srv.close()
    del other


def test_budget_admission_and_eviction(gpu):
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.server import Server
    srv = Server(gpu, budget_bytes=40 << 20, max_batch_views=4, streams=2)
    rng = np.random.default_rng(3)
    big = scenes.plain_large(2)  # its scratch and outputs alone (about 51 MB) exceed 40 MiB
    sid = srv.register(big.lights)
    rid = srv.submit(big.ubo, sid)
    c = take(srv, 1)[rid]
    assert c.status == 7  # CF_ERROR_BUDGET
    # many small sets: the oldest unused ones are evicted to make room
    small = [scenes.uniform_box_lights(rng, 60000, [-20, 0, -40], [20, 15, 10]) for _ in range(40)]
    ids = [srv.register(s) for s in small]
    assert srv.stats()["evictions"] > 0 and not srv.resident(ids[0]) and srv.resident(ids[-1])
    v = scenes.plain_small(1)
    with pytest.raises(CfError) as e:
        srv.submit(v.ubo, ids[0])  # evicted
    assert e.value.status == 5  # CF_ERROR_NOT_READY
    with pytest.raises(CfError):
        srv.register(np.zeros((2_000_000, 12), np.float32))  # larger than the whole budget
    srv.close()


def test_load_driver_completes_every_request(gpu):
    from hellovulkan_gb300.server import Server, run_load
    srv = Server(gpu, budget_bytes=4 << 30)
    rng = np.random.default_rng(9)
    base = [scenes.blob_lights(rng, int(n)) for n in (256, 1000, 4000, 12000)]
    rep = run_load(srv, rate=2000.0, duration=0.5, base_sets=base, submit_threads=2)
    assert rep["scheduled"] > 500 and rep["completed"] == rep["submitted"] and rep["failed"] == 0
    assert rep["latency_p50_ms"] > 0 and rep["latency_p99_ms"] >= rep["latency_p50_ms"]
    assert rep["reused_sets"] > 0 and rep["new_sets"] > 0
    srv.close()


def test_queued_jitters_chains_releases_and_idle_flush(gpu, oracle):
    """Jitters wait in the server's queue until the worker launches them (up
    to 32 sets per launch, a set whose source another queued jitter writes in
    a later launch): 40 sets jittered at once, one set jittered three times
    with a request after each step, a set released while its jitter waits,
    and a jitter flushed with no batch to carry it.  Every result matches the
    oracle on the host restatement of the jitter chain."""
    import time

    from hellovulkan_gb300.server import Server
    from oracle import jitter_lights
    srv = Server(gpu, budget_bytes=1 << 30, max_batch_views=16, streams=2)
    rng = np.random.default_rng(5)
    v = scenes.plain_small(4)
    sets = [scenes.uniform_box_lights(rng, int(n), [-20, -10, -60], [20, 10, -1], 1.0, 6.0)
            for n in rng.integers(1, 700, 40)]
    ids = [srv.register(s) for s in sets]
    expect = {}
    for k, (sid, s) in enumerate(zip(ids, sets)):
        srv.jitter(sid, 100 + k, 0.5)
        expect[srv.submit(v.ubo, sid)] = jitter_lights(s, 100 + k, 0.5)
    chain = jitter_lights(sets[0], 100, 0.5)  # set 0 again: each step reads the previous step's version
    for step in range(3):
        srv.jitter(ids[0], 7 + step, 0.25)
        chain = jitter_lights(chain, 7 + step, 0.25)
        expect[srv.submit(v.ubo, ids[0])] = chain
    gone = srv.register(sets[1])
    srv.jitter(gone, 99, 0.5)
    srv.release_set(gone)  # its queued jitter still holds both versions until launched
    extra = srv.register(sets[2])
    srv.jitter(extra, 55, 0.5)
    time.sleep(0.05)  # no request: the worker flushes the jitter alone
    expect[srv.submit(v.ubo, extra)] = jitter_lights(sets[2], 55, 0.5)
    done = take(srv, len(expect))
    for rid, lights in expect.items():
        assert done[rid].status == 0
        cells, idx = srv.read(done[rid])
        oc, oi = oracle_result(oracle, v.ubo, lights)
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi), rid
        srv.release(rid)
    srv.close()


def test_pinned_registers_and_updates_are_copied_by_the_worker(gpu, oracle):
    """From pinned memory a register or an update queues its copy: the worker
    reads the host buffers from the device (up to 48 per launch) ahead of the
    queued jitters and the next batch.  60 pinned sets at once, a jitter of a
    set whose copy is still queued, an update followed by a jitter, and a
    pinned buffer that is not 16-byte aligned (copied at once instead)."""
    torch = pytest.importorskip("torch")
    from hellovulkan_gb300.server import Server
    from oracle import jitter_lights
    srv = Server(gpu, budget_bytes=1 << 30, max_batch_views=8, streams=2)
    rng = np.random.default_rng(6)
    v = scenes.plain_small(5)
    sets = [np.ascontiguousarray(scenes.uniform_box_lights(rng, int(n), [-20, -10, -60], [20, 10, -1], 1.0, 6.0),
                                 np.float32) for n in rng.integers(1, 3000, 60)]
    pinned = [torch.from_numpy(s).pin_memory() for s in sets]
    ids = [srv.register(p.numpy()) for p in pinned]
    expect = {srv.submit(v.ubo, sid): s for sid, s in zip(ids, sets)}
    a = srv.register(pinned[0].numpy())
    srv.jitter(a, 3, 0.5)  # reads the version the queued copy writes
    expect[srv.submit(v.ubo, a)] = jitter_lights(sets[0], 3, 0.5)
    srv.update(ids[1], pinned[2].numpy())
    expect[srv.submit(v.ubo, ids[1])] = sets[2]
    srv.jitter(ids[1], 4, 0.5)
    expect[srv.submit(v.ubo, ids[1])] = jitter_lights(sets[2], 4, 0.5)
    flat = torch.empty(sets[3].size + 1, dtype=torch.float32).pin_memory()
    flat[1:] = torch.from_numpy(sets[3].reshape(-1))
    odd = flat[1:].numpy().reshape(-1, 12)  # 4 bytes past a 16-byte boundary
    assert odd.ctypes.data % 16 == 4
    b = srv.register(odd)
    expect[srv.submit(v.ubo, b)] = sets[3]
    done = take(srv, len(expect))
    for rid, lights in expect.items():
        assert done[rid].status == 0
        cells, idx = srv.read(done[rid])
        oc, oi = oracle_result(oracle, v.ubo, lights)
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi), rid
        srv.release(rid)
    srv.close()
    del pinned, flat


def test_failed_version_writes_fail_their_requests_and_nothing_else(gpu, oracle, cflib):
    """A queued jitter whose launch fails (a test hook fails it on the host,
    nothing is launched): the batch that carried it reports CF_ERROR_CUDA,
    later requests bound to the unwritten version (and to a jitter of it)
    fail at admission, the idle-flush path fails the same way, and a new
    version from the host brings the set back, bit-exact."""
    import time

    from hellovulkan_gb300.server import Server
    from oracle import jitter_lights
    CF_ERROR_CUDA = 3
    srv = Server(gpu, budget_bytes=256 << 20, streams=1)
    v = scenes.plain_small(9)
    sid = srv.register(v.lights)  # pageable: copied before the call returns

    def take(srv, count):
        out = srv.wait_all(count, timeout_s=10.0)
        assert len(out) == count, (srv.stats(), cflib.cf_last_error_message())
        return {c.request_id: c for c in out}

    try:
        rid = srv.submit(v.ubo, sid)
        assert take(srv, 1)[rid].status == 0
        srv.release(rid)
        cflib.cf_testing_fail_version_writes(1)
        srv.jitter(sid, 5, 0.5)
        carried = srv.submit(v.ubo, sid)  # its batch carries the failing launch
        assert take(srv, 1)[carried].status == CF_ERROR_CUDA
        later = srv.submit(v.ubo, sid)  # bound to the unwritten version
        assert take(srv, 1)[later].status == CF_ERROR_CUDA
        srv.jitter(sid, 6, 0.5)  # a jitter of it is unwritten too
        rid = srv.submit(v.ubo, sid)
        assert take(srv, 1)[rid].status == CF_ERROR_CUDA
        srv.update(sid, v.lights)  # a new version from the host
        cflib.cf_testing_fail_version_writes(1)
        srv.jitter(sid, 7, 0.5)
        time.sleep(0.05)  # no request: the idle flush fails
        rid = srv.submit(v.ubo, sid)
        assert take(srv, 1)[rid].status == CF_ERROR_CUDA
        srv.update(sid, v.lights)
        srv.jitter(sid, 8, 0.5)  # and works again
        rid = srv.submit(v.ubo, sid)
        c = take(srv, 1)[rid]
        assert c.status == 0
        cells, idx = srv.read(c)
        oc, oi = oracle_result(oracle, v.ubo, jitter_lights(v.lights, 8, 0.5))
        assert np.array_equal(cells, oc) and np.array_equal(idx, oi)
    finally:
        cflib.cf_testing_fail_version_writes(0)
        srv.close()
