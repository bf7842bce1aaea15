"""Path-replay gradients against central finite differences (needs a GB300).

Loss: mean squared error of sensor irradiance (rtrace -I, two ambient
bounces) to a target map made with other material colours, in a room with
a glass window and the glow sky.  Parameters: the RGB reflectances of the
triangle materials and the window's transmissivity.  The finite
differences use the same random streams (-u-, common random numbers) and
-lw small enough that no Russian roulette decision depends on the
parameters, so both estimate the derivative of the same fixed-seed
estimator; the bar is 1% of the derivative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARGS = ("-I+", "-ab", "2", "-ad", "64", "-aa", "0", "-as", "0", "-lw", "1e-6", "-u-")
NMAT = 8


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    torch = pytest.importorskip("torch")
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import workloads as w
    d = tmp_path_factory.mktemp("grad")
    rad = d / "room.rad"
    rad.write_text(w.window_room(seed=3, ntri=2000, nmat=NMAT))
    sc = gb.Scene(rad_files=[rad])
    rays = w.sensor_grid(16, 16)
    rng = np.random.default_rng(11)
    truth = {f"tri_mat{m}": torch.tensor(rng.uniform(0.2, 0.8, 3)) for m in range(NMAT)}
    truth["window_glass"] = torch.tensor([0.45])
    init = {f"tri_mat{m}": torch.tensor(rng.uniform(0.2, 0.8, 3)) for m in range(NMAT)}
    init["window_glass"] = torch.tensor([0.6])
    return torch, sc, rays, truth, init


def loss_of(torch, sc, rays, params, target):
    from pyradiance_gb300.grad import sensor_values
    e = sensor_values(sc, rays, params, ARGS)
    return ((e - target) ** 2).mean()


def test_gradient_matches_central_differences(setup):
    torch, sc, rays, truth, init = setup
    from pyradiance_gb300.grad import sensor_values
    with torch.no_grad():
        target = sensor_values(sc, rays, truth, ARGS)
    params = {k: v.clone().requires_grad_(True) for k, v in init.items()}
    loss = loss_of(torch, sc, rays, params, target)
    loss.backward()
    assert loss.item() > 0
    h = 1e-3
    checked = 0
    for name in ["tri_mat0", "tri_mat3", "tri_mat5", "window_glass"]:
        for ch in range(params[name].numel()):
            g_ad = params[name].grad[ch].item()
            vals = []
            for sgn in (1, -1):
                p = {k: v.detach().clone() for k, v in init.items()}
                p[name][ch] += sgn * h
                with torch.no_grad():
                    vals.append(loss_of(torch, sc, rays, p, target).item())
            g_fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(g_ad - g_fd) <= 0.01 * abs(g_fd) + 1e-9, (name, ch, g_ad, g_fd)
            checked += 1
    assert checked == 10


def test_gradient_of_total_irradiance_is_nonnegative(setup):
    """Every path coefficient grows with each reflectance and with the
    glass transmissivity (both glass coefficients increase with it), so the
    gradient of the summed irradiance is finite and non-negative."""
    torch, sc, rays, truth, init = setup
    from pyradiance_gb300.grad import sensor_values
    params = {k: v.clone().requires_grad_(True) for k, v in init.items()}
    s = sensor_values(sc, rays, params, ARGS).sum()
    s.backward()
    for k, v in params.items():
        assert torch.isfinite(v.grad).all(), k
        assert (v.grad >= 0).all(), (k, v.grad)       # more reflectance or transmission, more light


# -lw 1e-6: at -lw 1e-4 some paths end or continue depending on their
# weights, which the parameters move, so a central difference with common
# random numbers no longer differentiates one fixed estimator (4.5% off for
# one of the smallest components measured); at 1e-6 no path's fate depends
# on the parameters at two bounces
C4_ARGS = ("-I+", "-ab", "2", "-ad", "1024", "-aa", "0", "-as", "0", "-lw", "1e-6", "-u-")


@pytest.fixture(scope="module")
def c4(tmp_path_factory):
    """The gradient workload: the window room with its 20,000 triangles in
    64 plastic materials and the glass window, 4,096 sensors (64 x 64),
    -ab 2 -ad 1024; reflectances initialised U[0.2, 0.8], the target map
    made by a seed-fixed ground-truth parameter set."""
    torch = pytest.importorskip("torch")
    import pyradiance_gb300 as gb
    from pyradiance_gb300 import workloads as w
    d = tmp_path_factory.mktemp("c4")
    rad = d / "room64.rad"
    rad.write_text(w.window_room(seed=0, ntri=20000, nmat=64))
    sc = gb.Scene(rad_files=[rad])
    rng = np.random.default_rng(2024)
    truth = {f"tri_mat{m}": torch.tensor(rng.uniform(0.2, 0.8, 3)) for m in range(64)}
    truth["window_glass"] = torch.tensor([0.5])
    init = {f"tri_mat{m}": torch.tensor(rng.uniform(0.2, 0.8, 3)) for m in range(64)}
    init["window_glass"] = torch.tensor([0.6])
    names = [f"tri_mat{m}" for m in range(64)] + ["window_glass"]
    text = {nm: sc.material_rgb(sc.material_slot(nm)).copy() for nm in names}
    return torch, sc, w.sensor_grid(64, 64), truth, init, text


def test_c4_gradient_matches_central_differences(c4):
    """MSE loss over 4,096 sensor irradiances; the path-replay gradient of
    eight material channels and the glass transmissivity against central
    differences (step 1e-3, common random numbers) within 1%."""
    torch, sc, rays, truth, init, _ = c4
    from pyradiance_gb300.grad import sensor_values
    with torch.no_grad():
        target = sensor_values(sc, rays, truth, C4_ARGS)
    params = {k: v.clone().requires_grad_(True) for k, v in init.items()}
    loss = ((sensor_values(sc, rays, params, C4_ARGS) - target) ** 2).mean()
    loss.backward()
    h = 1e-3
    picks = [("tri_mat0", 0), ("tri_mat9", 1), ("tri_mat17", 2), ("tri_mat23", 0), ("tri_mat31", 1),
             ("tri_mat42", 2), ("tri_mat55", 0), ("tri_mat63", 1), ("window_glass", 0)]
    worst = 0.0
    for name, ch in picks:
        g_ad = params[name].grad[ch].item()
        vals = []
        for sgn in (1, -1):
            p = {k: v.detach().clone() for k, v in init.items()}
            p[name][ch] += sgn * h
            with torch.no_grad():
                vals.append(((sensor_values(sc, rays, p, C4_ARGS) - target) ** 2).mean().item())
        g_fd = (vals[0] - vals[1]) / (2 * h)
        rel = abs(g_ad - g_fd) / abs(g_fd)
        worst = max(worst, rel)
        assert rel <= 0.01, (name, ch, g_ad, g_fd)
    print("C4 gradient vs central differences: worst relative difference %.2e" % worst)


def test_gradient_matches_differenced_reference_runs(c4):
    """The derivative of the mean red irradiance of 1,024 sensors with
    respect to three materials' reflectances and the window's
    transmissivity: the path-replay gradient (mean of 8 seeds) against the
    reference's central differences (rtrace -u-, common random numbers,
    tests/golden/grad_fd.npz), at the colours of the scene text.  Both are
    Monte Carlo estimates of the same derivative: the reference's is one
    realisation, whose spread is that of one seed of ours (the same
    sampling of the same paths), so the bound is four times the combined
    spread of our mean and one seed, with a floor of 1% of the
    derivative."""
    torch, sc, _, _, _, text = c4
    from conftest import golden
    from pyradiance_gb300 import _lib
    g = golden("grad_fd.npz")
    for nm, rgb in text.items():
        sc.material_rgb(sc.material_slot(nm), rgb)
    rays = np.ascontiguousarray(g["rays"])
    n = len(rays)
    dl = np.zeros((n, 3))
    dl[:, 0] = 1.0 / n
    ns = int(_lib.lib().gb_scene_material_slots(sc.handle))
    ests = []
    for seed in range(8):
        o, _ = _lib.parse_opts(["-I", "-ab", "2", "-ad", "1024", "-aa", "0", "-as", "0", "-lw", "1e-6"],
                               _lib.GB_PROG_RTRACE)
        o.u, o.seed = 0, 1000 + seed
        grad = np.zeros((ns, 3))
        _lib.check(_lib.lib().gb_rtrace_grad(sc.handle, o, _lib.ptr(rays), n, _lib.ptr(dl), _lib.ptr(grad), ns))
        ests.append([grad[sc.material_slot(str(nm)), 0] for nm in g["names"]])
    ests = np.array(ests)
    ours, ours_se = ests.mean(0), ests.std(0, ddof=1) / np.sqrt(len(ests))
    ref = g["fd"][:, :, 0].mean(1)
    ref_se = ests.std(0, ddof=1)                     # one realisation's spread
    for k, nm in enumerate(g["names"]):
        tol = max(4 * np.hypot(ours_se[k], ref_se[k]), 0.01 * abs(ref[k]))
        print("%s: path replay %.5g +- %.2g, reference differences %.5g" % (nm, ours[k], ours_se[k], ref[k]))
        assert abs(ours[k] - ref[k]) <= tol, (nm, ours[k], ref[k], tol)
