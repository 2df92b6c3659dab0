"""Host side of the selection and auto-SPP rows: the C auto-SPP controller (vkrt_host_auto_spp_*, restating
src/core/scene/timing.c:121-178 and api/settings.c:68-79) against the oracle's float32 restatement, and the outline
oracle against hand-worked masks."""
import numpy as np
import pytest

from oracle import overlay
from vkrt_gb300.context import AutoSpp


@pytest.mark.parametrize("fps", [0, 10, 60, 144, 1000])
def test_auto_spp_target_clamp(built, fps):
    c = AutoSpp(fps)
    want = overlay.auto_spp_init(fps)["targetFrameMs"]
    assert c.target_ms == float(want)
    assert 1000.0 / 360 - 1e-4 <= c.target_ms <= 1000.0 / 30 + 1e-4


@pytest.mark.parametrize("seed", range(6))
def test_auto_spp_controller_matches_oracle(built, seed):
    """Random frame-time sequences (noisy linear cost per sample, occasional spikes and zero readings): the C
    controller's spp sequence and smoothed state are identical to the oracle's."""
    rng = np.random.default_rng(seed)
    fps = int(rng.choice([30, 60, 120, 240]))
    c, o = AutoSpp(fps), overlay.auto_spp_init(fps)
    spp_c = spp_o = int(rng.integers(0, 4))
    base, per = rng.uniform(0.1, 2.0), rng.uniform(0.01, 1.5)
    for i in range(300):
        ms = float(np.float32(base + per * max(spp_c, 1) * rng.uniform(0.8, 1.25)))
        if rng.uniform() < 0.05:
            ms *= 8.0
        if rng.uniform() < 0.02:
            ms = 0.0
        spp_c = c.update(ms, spp_c)
        spp_o = overlay.auto_spp_update(o, ms, spp_o)
        assert spp_c == spp_o, (i, spp_c, spp_o)
        assert c.state["controlMs"][0] == o["controlMs"]
        assert 0 <= spp_c <= 2048


def test_auto_spp_converges_to_budget(built):
    """A noiseless cost model ms = 1 + 0.25 spp at 60 FPS settles inside the deadband below 90% of 16.7 ms."""
    c = AutoSpp(60)
    spp = 1
    for _ in range(60):
        spp = c.update(1.0 + 0.25 * spp, spp)
    ms = 1.0 + 0.25 * spp
    assert 0.7 * 15.0 <= ms <= 15.0 + 0.25, (spp, ms)


def test_outline_oracle_square_ring():
    """One selected pixel on a 1080 x 1080 film (radius 2): exactly the 5 x 5 square around it minus the pixel."""
    h, w = 1080, 1080
    mask = np.zeros((h, w), np.uint32)
    mask[500, 20] = 1
    out = overlay.outline(mask, np.zeros((h, w, 4), np.uint16))
    painted = np.argwhere(out[..., 0] == 65535)
    assert len(painted) == 24
    assert painted[:, 0].min() == 498 and painted[:, 0].max() == 502
    assert painted[:, 1].min() == 18 and painted[:, 1].max() == 22
    assert out[500, 20, 0] == 0


@pytest.mark.parametrize("size,radius", [((64, 64), 1), ((1920, 1080), 2), ((3840, 2160), 4), ((8000, 6000), 5),
                                         ((1350, 1350), 2), ((810, 900), 2)])
def test_outline_radius(size, radius):
    assert overlay.outline_radius(*size) == radius
