"""Render export (vkrt_gb300.image_io, following src/core/utility/export/image.c): PNG and EXR round trips, the
spectral XYZ -> linear sRGB conversion, and the display encode against the oracle's restatement of vkrt's tone map
on a rendered frame."""
import numpy as np
import pytest

from vkrt_gb300 import abi, image_io, scenes


def test_png16_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 65536, size=(37, 53, 4), dtype=np.uint16)
    image_io.write_png16(tmp_path / "a.png", img)
    np.testing.assert_array_equal(image_io.read_png16(tmp_path / "a.png"), img)


def test_exr_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.normal(size=(19, 31, 4)).astype(np.float32) * 100
    image_io.write_exr(tmp_path / "a.exr", img)
    np.testing.assert_array_equal(image_io.read_exr(tmp_path / "a.exr"), img)


def test_spectral_white_maps_to_srgb_white(built):
    """Equal-energy XYZ (1, 1, 1) adapts to D65 and converts to linear sRGB (1, 1, 1)."""
    sd = scenes.default_scene_data(4, 4)
    sd["packedRenderSettings"] = abi.pack_render_settings(1, abi.RENDER_MODE_SPECTRAL, 1)
    lin = image_io.linear_rgba(np.ones((2, 2, 4), np.float32), sd)
    np.testing.assert_allclose(lin[..., :3], 1.0, atol=2e-3)
    np.testing.assert_array_equal(lin[..., 3], 1.0)
    bad = np.full((1, 1, 4), np.nan, np.float32)
    sd["packedRenderSettings"] = abi.pack_render_settings(1, abi.RENDER_MODE_RGB, 1)
    assert np.all(image_io.linear_rgba(bad, sd)[..., :3] == 0.0)


@pytest.mark.parametrize("tone", [0, 1])
def test_display_encode_matches_oracle_tone_map(built, tone):
    """The export's display image of an oracle-rendered Cornell frame equals the oracle's tone-mapped output
    (tonemap.slang) to one unit in the last place of 16 bits."""
    from oracle import cpu
    s = scenes.cornell(48, 48, spp=2)
    sd = s.scene_data.copy()
    sd["packedRenderSettings"] = abi.pack_render_settings(tone, abi.RENDER_MODE_RGB, 1)
    sd["exposure"] = 1.7
    acc, out, _ = cpu.OracleScene(s).render(sd, want_output=True)
    disp = image_io.display_rgba16(image_io.linear_rgba(acc, sd), sd)
    assert np.abs(disp.astype(np.int64) - out.astype(np.int64)).max() <= 1


def test_export_render(built, tmp_path):
    sd = scenes.default_scene_data(8, 6)
    acc = np.random.default_rng(2).uniform(0, 3, size=(6, 8, 4)).astype(np.float32)
    image_io.export_render(tmp_path / "r.exr", acc, sd)
    np.testing.assert_array_equal(image_io.read_exr(tmp_path / "r.exr")[..., :3], acc[..., :3])
    image_io.export_render(tmp_path / "r.png", acc, sd)
    np.testing.assert_array_equal(image_io.read_png16(tmp_path / "r.png"),
                                  image_io.display_rgba16(image_io.linear_rgba(acc, sd), sd))
    with pytest.raises(ValueError):
        image_io.export_render(tmp_path / "r.jpg", acc, sd)
