"""The in-process simulation managers with pyradiance's binding API
(src/binding/radiance_ext.cpp:170-458, tests/test_rtrace.py and
tests/test_rcontrib.py of the reference) on the GPU."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _restore_params():
    import pyradiance_gb300 as pr
    yield
    pr.set_ray_params()


def test_rtrace_simul_manager_callbacks(scene_dir):
    """Two rays, cooked and trace callbacks (the reference's test: four
    results), then the C1 sensors with RTimmIrrad: every callback in ray
    order with the reference's irradiance (1e-5) and ray numbers."""
    import pyradiance_gb300 as pr
    rp = pr.get_ray_params()
    rp.ab = 0
    pr.set_ray_params(rp)
    result = []
    mgr = pr.RtraceSimulManager()
    mgr.load_octree(scene_dir / "c1.rad")
    assert mgr.ready() and mgr.set_thread_count(1) >= 1
    mgr.set_cooked_call(lambda ray, cd: result.append(ray.rcol) or 0)
    mgr.set_trace_call(lambda ray, cd: result.append(ray.rcol) or 0)
    mgr.rt_flags = pr.RTdoFIFO
    mgr.enqueue_bundle(np.array([[1.0, 2.0, 2.0], [0, 0, 1], [4.0, 5.0, 2.0], [0, 1, 0]]))
    mgr.flush_queue()
    assert len(result) == 4
    mgr.cleanup_callbacks()

    g = golden("c1_direct.npz")
    rp.dj, rp.ds, rp.dr, rp.u = 0.0, 0.0, 0, False
    pr.set_ray_params(rp)
    got = []
    mgr.set_cooked_call(lambda ray, cd: got.append((ray.rno, ray.rcol, ray.ro)) or 0)
    mgr.rt_flags = pr.RTdoFIFO | pr.RTimmIrrad
    rays = g["rays"]
    half = len(rays) // 2
    mgr.enqueue_bundle(rays[:half].reshape(-1, 3), rID0=1)
    mgr.enqueue_bundle(rays[half:].reshape(-1, 3), rID0=half + 1)
    assert mgr.flush_queue() == len(rays)
    assert [r[0] for r in got] == list(range(1, len(rays) + 1))
    rgb = np.array([r[1] for r in got])
    ref = g["irradiance"]
    lit = ref[:, 0] > 0
    np.testing.assert_array_equal(rgb[~lit], 0.0)
    assert (np.abs(rgb[lit] - ref[lit]) / ref[lit]).max() < 1e-5
    mgr.cleanup(True)
    assert not mgr.ready()


def test_rcontrib_simul_manager(scene_dir, tmp_path, monkeypatch):
    """The reference's RcontribSimulManager test on the window room: ground
    and Reinhart sky modifiers into one output file, -I sensors, fixed
    seeding; the records equal Rcontrib's for the same parameters, and the
    output file holds them with the matrix header."""
    import pyradiance_gb300 as pr
    monkeypatch.chdir(tmp_path)
    rp = pr.get_ray_params()
    rp.u, rp.ab, rp.ad, rp.lw, rp.aa, rp.as_ = False, 1, 64, 1e-3, 0.0, 0
    pr.set_ray_params(rp)
    rng = np.random.default_rng(3)
    sens = np.hstack([rng.uniform((1, 1, .8), (9, 7, .8), size=(64, 3)), np.tile([0.0, 0, 1], (64, 1))])
    params = "MF=1,rNx=0,rNy=0,rNz=-1,Ux=0,Uy=1,Uz=0,RHS=+1"
    pr.loadfunc("reinhartb.cal")
    with pr.RcontribSimulManager() as mgr:
        mgr.accum = 1
        mgr.yres = len(sens)
        mgr.set_flag(pr.RTimmIrrad, True)
        assert mgr.has_flag(pr.RTimmIrrad)
        mgr.add_modifier(modn="groundglow", outspec="test.mtx", binval="if(-Dx*0-Dy*0-Dz*-1,0,-1)", bincnt=1)
        mgr.add_modifier(modn="skyglow", outspec="test.mtx", prms=params, binval="rbin", bincnt=145)
        mgr.load_octree(scene_dir / "c2.rad")
        mgr.out_op = pr.RcOutputOp.FORCE
        assert mgr.prep_output() == 3 * 146
        assert mgr.rcontrib(sens.reshape(-1, 3)) == len(sens)
        arr = mgr.get_output_array()
        assert arr.shape == (len(sens), 146 * 3) and arr.sum() > 0
        rc = pr.Rcontrib(b"", scene_dir / "c2.rad", params=rp.args() + ["-I+", "-c", "1"])
        rc.add_modifier("groundglow", binv="if(-Dx*0-Dy*0-Dz*-1,0,-1)", nbins="1")
        rc.add_modifier("skyglow", calfile="reinhartb.cal", param=params, binv="rbin", nbins="145")
        np.testing.assert_array_equal(arr, rc.run_array(sens).reshape(len(sens), -1))
    data = (tmp_path / "test.mtx").read_bytes()
    head, body = data.split(b"\n\n", 1)
    assert b"NROWS=64" in head and b"NCOLS=146" in head and b"FORMAT=float" in head
    np.testing.assert_allclose(np.frombuffer(body, dtype="<f4").reshape(64, -1), arr, rtol=1e-6)
