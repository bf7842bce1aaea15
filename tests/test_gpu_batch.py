"""gb_rcontrib_batch: many grids over several scenes in one call (needs a
GB300).  A job alone on its scene draws the same random streams as its
separate gb_rcontrib call, and jobs sharing a scene draw those of their
position in the scene's concatenated sensors, so the results reproduce the
corresponding separate calls up to rounding: the queue order, and with it
which lanes of a warp sum their FP32 contributions before the FP64 bin
atomics, differs from run to run (1e-6 relative)."""
import numpy as np
import pytest

from conftest import MODS_C2

pytestmark = pytest.mark.gpu

ARGS = ["-I+", "-ab", "2", "-ad", "256", "-lw", "1e-4", "-c", "1", "-u-"]


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import workloads as w
    d = tmp_path_factory.mktemp("batch")
    scenes = []
    for k, nt in enumerate((3000, 6000)):
        p = d / f"room{k}.rad"
        p.write_text(w.window_room(seed=k, ntri=nt))
        scenes.append(gb.Scene(rad_files=[p]))
    return gb, scenes


def rc_for(gb):
    rc = gb.Rcontrib(b"", None, params=ARGS)
    for m in MODS_C2:
        rc.add_modifier(**{{"expr": "expression", "params": "param"}.get(k, k): v for k, v in m.items()})
    rc.seed = 1234
    return rc


def grid(n, seed):
    rng = np.random.default_rng(seed)
    xy = rng.uniform((0.5, 0.5), (9.5, 7.5), size=(n, 2))
    return np.column_stack([xy, np.full(n, 0.8), np.zeros(n), np.zeros(n), np.ones(n)])


def test_single_job_per_scene_reproduces_separate_calls(setup):
    gb, scenes = setup
    rc = rc_for(gb)
    jobs = [(scenes[0], grid(37, 1)), (scenes[1], grid(200, 2))]
    outs = rc.run_batch(jobs)
    for (sc, r), o in zip(jobs, outs):
        rc.octree = sc
        ref = rc.run_array(r)
        assert o.shape == ref.shape
        np.testing.assert_allclose(o, ref, rtol=1e-6, atol=1e-12)


def test_jobs_sharing_a_scene(setup):
    gb, scenes = setup
    rc = rc_for(gb)
    big = grid(1500, 3)
    jobs = [(scenes[0], big[:700]), (scenes[1], grid(64, 4)), (scenes[0], big[700:])]
    outs = rc.run_batch(jobs)
    assert [o.shape[0] for o in outs] == [700, 64, 800]
    rc.octree = scenes[0]
    ref = rc.run_array(big)
    got = np.concatenate([outs[0], outs[2]])
    # same sensors, same seed, same stream positions: the concatenation of
    # the two jobs is the separate call over all 1,500 sensors
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-12)
    assert rc.last_rays > 0


def test_tuned_graph_batch_equals_host_loop(setup, monkeypatch):
    """A job of more than 4,096 sensors runs the scene's tuner (queue size
    and walk shape from pilot runs) and its generation loop as a CUDA
    graph; the same batch with the host-driven loop (GB_GRAPHS=0) and the
    separate call give the same bins up to rounding."""
    gb, scenes = setup
    rc = rc_for(gb)
    big = grid(6000, 5)
    jobs = [(scenes[1], big), (scenes[0], grid(300, 6))]
    graph = rc.run_batch(jobs)
    monkeypatch.setenv("GB_GRAPHS", "0")
    host = rc.run_batch(jobs)
    for a, b in zip(graph, host):
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-12)
    monkeypatch.delenv("GB_GRAPHS")
    rc.octree = scenes[1]
    np.testing.assert_allclose(graph[0], rc.run_array(big), rtol=1e-6, atol=1e-12)
