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
