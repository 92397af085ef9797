"""Randomised operation sequences against the culling server, checked against
the oracle on a host model of every light set's versions.

Each sequence draws registers and updates (from pageable memory, from pinned
memory, and from a declared pinned pool), jitters, releases and submissions
over a handful of sets, with polls in between, under a budget small enough
that sets get evicted.  Copy on write means a request's result depends only
on the version its set had when it was submitted; the model records that
version (jitters restated on the host), and every completed request must
equal the oracle on it bit for bit.  An operation on an evicted set must
report CF_ERROR_NOT_READY, after which the model forgets the set; one that
finds no room for a new version reports CF_ERROR_BUDGET and leaves the set
as it was.  Completions are checked and released as they are polled."""
import numpy as np
import pytest

from hellovulkan_gb300 import scenes

pytestmark = pytest.mark.gpu

CF_ERROR_NOT_READY, CF_ERROR_BUDGET = 5, 7


def oracle_result(oracle, ubo, lights, cap=150):
    a = oracle.generate_aabbs(ubo)
    cells, idx, _ = oracle.cull(ubo, a, lights, cap)
    return cells, idx


@pytest.mark.parametrize("seed,budget_mb,streams", [(31, 16, 2), (32, 256, 4), (33, 12, 1)])
def test_random_server_sequences(gpu, oracle, seed, budget_mb, streams):
    torch = pytest.importorskip("torch")
    from hellovulkan_gb300 import CfError
    from hellovulkan_gb300.server import Server
    from oracle import jitter_lights
    rng = np.random.default_rng(seed)
    srv = Server(gpu, budget_bytes=budget_mb << 20, max_batch_views=int(rng.integers(1, 17)), streams=streams)
    views = [scenes.plain_small(s) for s in (3, 4)] + [
        scenes.custom_view((15, 9, 7), 1280, 720, 0.1, 300.0, view=scenes.random_camera(rng))]
    pool = torch.from_numpy(np.ascontiguousarray(
        scenes.uniform_box_lights(rng, 24000, [-20, -10, -60], [20, 10, -1], 1.0, 6.0), np.float32)).pin_memory()
    srv.declare_pinned(pool)
    keep = [pool]  # pinned sources stay allocated and unchanged to the end

    def source(n):
        kind = int(rng.integers(0, 3))
        if kind == 0:  # pageable: copied before the call returns
            return scenes.uniform_box_lights(rng, n, [-20, -10, -60], [20, 10, -1], 1.0, 6.0)
        if kind == 1:  # pinned, undeclared
            t = torch.from_numpy(np.ascontiguousarray(
                scenes.uniform_box_lights(rng, n, [-20, -10, -60], [20, 10, -1], 1.0, 6.0), np.float32)).pin_memory()
            keep.append(t)
            return t.numpy()
        start = int(rng.integers(0, pool.shape[0] - n))  # a slice of the declared pool
        return pool.numpy()[start:start + n]

    model = {}  # set id -> its current lights
    expect = {}  # request id -> (view, lights it bound)
    checked = 0

    def check(completions):
        nonlocal checked
        for c in completions:  # checked and released at once: held outputs take budget
            v, lights = expect.pop(c.request_id)
            assert c.status == 0, (c.request_id, c.status)
            cells, idx = srv.read(c)
            oc, oi = oracle_result(oracle, v.ubo, lights)
            assert np.array_equal(cells, oc) and np.array_equal(idx, oi), c.request_id
            srv.release(c.request_id)
            checked += 1

    for _ in range(400):
        op = rng.random()
        sid = None
        try:
            if op < 0.18 or not model:
                lights = source(int(rng.integers(1, 1500)))
                sid = srv.register(lights)
                model[sid] = np.array(lights, copy=True)
            elif op < 0.30:
                sid = int(rng.choice(list(model)))
                lights = source(int(rng.integers(1, 1500)))
                srv.update(sid, lights)
                model[sid] = np.array(lights, copy=True)
            elif op < 0.50:
                sid = int(rng.choice(list(model)))
                s, sigma = int(rng.integers(0, 1 << 30)), float(rng.uniform(0.05, 1.0))
                srv.jitter(sid, s, sigma)
                model[sid] = jitter_lights(model[sid], s, sigma)
            elif op < 0.56:
                sid = int(rng.choice(list(model)))
                srv.release_set(sid)
                del model[sid]
            else:
                sid = int(rng.choice(list(model)))
                v = views[int(rng.integers(0, len(views)))]
                expect[srv.submit(v.ubo, sid)] = (v, model[sid])
        except CfError as e:
            if e.status == CF_ERROR_NOT_READY:  # the set was evicted to make room
                model.pop(sid, None)
            else:  # no room for a new version right now: the set keeps its old one
                assert e.status == CF_ERROR_BUDGET, e
        if rng.random() < 0.2:
            check(srv.poll(wait_ms=0))
    while expect:
        got = srv.wait_all(1, timeout_s=30.0)
        assert got, "requests did not complete"
        check(got)
    evictions = srv.stats()["evictions"]
    srv.close()
    assert checked > 100
    assert budget_mb > 100 or evictions > 0, evictions  # the small budgets did evict sets
