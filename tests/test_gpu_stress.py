"""GPU tests of the animated many-view workload: the in-place orbit animation
bit for bit against its host restatement, the batched AABB generator against
the oracle, and a short animated run whose sampled frames match the oracle
across projection changes."""
import numpy as np
import pytest

from hellovulkan_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_orbit_animation_matches_the_host_restatement(gpu):
    import torch
    from hellovulkan_gb300._lib import check, lib
    from oracle import animate_orbits
    rng = np.random.default_rng(11)
    lights, orbits = scenes.orbit_lights(rng, 3, 3333)  # 9999 lights: not a multiple of the block size
    d_l, d_o = torch.from_numpy(lights).cuda(), torch.from_numpy(orbits).cuda()
    done = 0
    for frames in (1, 0, 7, 60):
        check(lib().cf_animate_light_orbits(d_l.data_ptr(), d_o.data_ptr(), lights.shape[0], frames, None))
        done += frames
        torch.cuda.synchronize()
        o, pos = animate_orbits(orbits, done)
        got_l, got_o = d_l.cpu().numpy(), d_o.cpu().numpy()
        assert np.array_equal(got_o.view(np.uint32), o.view(np.uint32))
        assert np.array_equal(got_l[:, :4].view(np.uint32), pos.view(np.uint32))
        assert np.array_equal(got_l[:, 4:].view(np.uint32), lights[:, 4:].view(np.uint32))  # colour, radius


def test_batched_aabbs_match_the_oracle(gpu, oracle):
    import torch
    from hellovulkan_gb300.batch import Batch, BatchBuffers
    rng = np.random.default_rng(12)
    views = [scenes.batch_view(rng, scenes.blob_lights(rng, 300)) for _ in range(9)]
    bufs = BatchBuffers(views)
    b = Batch(gpu)
    b.set_views(bufs.batch_views())
    b.generate_aabbs(None)
    torch.cuda.synchronize()
    for i, v in enumerate(views):
        got = bufs.aabbs[i].cpu().numpy().reshape(v.clusters, 8)
        assert np.array_equal(got.view(np.uint32), oracle.generate_aabbs(v.ubo).view(np.uint32))
    b.close()


def test_animated_views_match_the_oracle_across_projection_changes(gpu, oracle):
    import torch
    from hellovulkan_gb300.stress import StressAnimation
    st = StressAnimation(gpu, n_views=8, n_lights=700, seed=13, frames_per_projection=5)
    stream = torch.cuda.Stream()
    # the epoch at frame 5 follows a check (the device is idle), the one at
    # frame 10 follows unchecked frames still queued on the stream
    from bench import check_stress_view
    rep = st.run(12, stream, check_frames={0, 4, 5, 7, 11}, check_views=(0, 3, 6),
                 check=lambda state: check_stress_view(state, oracle))
    st.close()
    assert len(rep["checks"]) == 15
    bad = [c for c in rep["checks"] if not all(c[k] for k in ("lights", "aabbs", "cells", "indices"))]
    assert not bad, bad
    assert rep["parity"] and len(rep["projection_frame_ms"]) == 3
    assert gpu.check_device_error() == 0
