"""bench.py's CPU arms (the reference arm and cpu_baseline) on the host: repeated calls on one scene render the
same spectral frame (the arm times several steps of it), and the oracle refuses a spectral frame whose rgb2spec
layout does not fit its table instead of reading past it."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))


def test_cpu_baseline_leaves_the_scene_unchanged():
    import bench
    from vkrt_gb300 import scenes
    scene = scenes.icosphere_field(n_spheres=20, width=64, height=1080, spp=1, max_depth=3, seed=1, spectral=True)
    for _ in range(2):
        r = bench.cpu_baseline(scene, budget_s=0.05, threads=2)
        assert r["value"] > 0 and scene.rgb2spec is None


def test_oracle_refuses_a_table_smaller_than_its_layout():
    from oracle import cpu
    from vkrt_gb300 import abi, scenes
    s = scenes.cornell(8, 8, spp=1)
    s.rgb2spec = cpu.rgb2spec_generate(8)
    s.scene_data["packedRenderSettings"] = abi.pack_render_settings(abi.TONE_MAPPING_ACES, abi.RENDER_MODE_SPECTRAL,
                                                                     abi.SPECTRAL_HERO)
    s.scene_data["rgb2specSRGB"] = (64, 0, 64)  # the layout of a 64-entry table
    with pytest.raises(RuntimeError):
        cpu.OracleScene(s).render(s.scene_data)
    s.scene_data["rgb2specSRGB"] = (8, 0, 8)
    img, _ = cpu.OracleScene(s).render(s.scene_data)
    assert np.isfinite(img).all()
