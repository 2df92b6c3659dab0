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
    from oracle.host import OracleHost
    scene = scenes.icosphere_field(n_spheres=20, width=64, height=1080, spp=1, max_depth=3, seed=1, spectral=True,
                                   host=OracleHost)
    for k in range(2):
        r = bench.cpu_baseline(scene, budget_s=0.05, threads=2, offset=k, rgb2spec_res=8)
        assert r["value"] > 0 and scene.rgb2spec is None
        assert 0 < r["frame_fraction"] <= 1 and r["samples_per_s"] > 0


def test_reference_arm_loads_no_product_library(tmp_path):
    """The reference arm's scenes come from the oracle's host layer: its process never maps libvkrt_gb300.so."""
    import subprocess
    code = ("import sys; sys.path.insert(0, '.'); import bench; from oracle.host import OracleHost; "
            "s = bench.build_scene(width=64, height=64, n_spheres=10, host=OracleHost); "
            "r = bench.cpu_baseline(s, budget_s=0.05, threads=2, rgb2spec_res=8); "
            "print(sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l}))")
    out = subprocess.run([sys.executable, "-c", code], cwd=Path(__file__).resolve().parents[1], capture_output=True,
                         text=True, check=True).stdout
    assert "liboracle.so" in out and "libvkrt_gb300.so" not in out, out


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


def test_clock_sampler_keeps_the_samples_of_the_timed_region(tmp_path, monkeypatch):
    """The clock record comes from samples taken while the timed region runs: a stand-in nvidia-smi on PATH prints
    a sample every 50 ms; start() returns once one has arrived and stop() parses the ones after it."""
    import os
    import time
    import bench
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\nwhile true; do\n"
                    "  echo '0, 1965, 2070, 700.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active'\n"
                    "  sleep 0.05\ndone\n")
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    sampler = bench.ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    r = sampler.stop()
    assert r["samples"] >= 3
    assert r["sm_mhz"] == 1965.0 and r["sm_max_mhz"] == 2070.0 and r["reasons"] == ["sw_power_cap"]
