"""Host-side scene compilation (no GPU): the compiled device scene passes index validation and the
light tree matches the oracle's ManyLightSampler build."""
import re

import numpy as np
import pytest

from lambda_gb300 import configs


@pytest.fixture(scope="module")
def lg():
    import lambda_gb300 as lg
    lg.build()
    return lg


CASES = {
    "cornell": lambda: configs.cornell(32, 32, 4),
    "terrain_small": lambda: configs.terrain(64, 36, 4, grid=96, n_emitters=300),
    "volume_small": lambda: configs.volume(48, 27, 4, n_instances=40, sphere_res=(24, 24)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_scene_compiles_and_validates(lg, name):
    sb, cam, opts = CASES[name]()
    rc, rep = lg.scene_check(sb)
    assert rc == 0, rep
    assert rep.startswith("ok"), rep


@pytest.mark.parametrize("name", ["cornell", "terrain_small", "volume_small"])
def test_light_tree_power_matches_oracle(lg, name):
    from oracle.oracle import Oracle
    sb, cam, opts = CASES[name]()
    rc, rep = lg.scene_check(sb)
    assert rc == 0, rep
    tp = float(re.search(r"tree_power=([0-9.eE+-]+)", rep).group(1))
    info = Oracle(sb).tree_info()
    assert tp == pytest.approx(info["tree_power"], rel=1e-6)


def test_bad_scene_rejected(lg):
    sb, cam, opts = configs.cornell(8, 8, 1)
    sb.objects[0] = (sb.objects[0][0], sb.objects[0][1], 999, sb.objects[0][3])   # material out of range
    rc, rep = lg.scene_check(sb)
    assert rc != 0 and "material" in rep


def test_unsupported_node_rejected(lg):
    """MicrofacetBTDF has no reference implementation: rejected with a clear status."""
    sb, cam, opts = configs.cornell(8, 8, 1)
    bx = sb.node("BXDF_MICROFACET_T", [0, 1.5], {0: (0.9, 0.9, 0.9, 1), 1: 0.2})
    sb.materials[0] = (bx, -1, -1, -1)
    rc, rep = lg.scene_check(sb)
    assert rc != 0 and "unsupported" in rep


def test_image_texture_needs_a_scene_texture(lg):
    sb, cam, opts = configs.cornell(8, 8, 1)
    tex = sb.node("IMAGE_TEXTURE", [3])       # no texture 3 in the scene
    bx = sb.node("BXDF_LAMBERTIAN", inputs={0: lg.out(tex)})
    sb.materials[0] = (bx, -1, -1, -1)
    rc, rep = lg.scene_check(sb)
    assert rc != 0 and "texture" in rep


def test_image_texture_scene_compiles(lg):
    sb, cams, opts = configs.cornell_inverse(16, 16, 1, tex_res=8)
    rc, rep = lg.scene_check(sb)
    assert rc == 0, rep


@pytest.mark.parametrize("kind", ["disc", "zero", "one_texel", "negative"])
def test_aperture_mask_textures_compile(lg, kind):
    """Masked-aperture distributions are built at commit for flagged textures, including an
    all-zero mask (uniform fallback of Piecewise1D), a 1x1 mask and negative red (|red|)."""
    sb, cam, opts = configs.cornell(8, 8, 1)
    if kind == "one_texel":
        m = np.ones((1, 1, 4), np.float32)
    else:
        yy, xx = np.mgrid[0:12, 0:9]
        m = np.zeros((12, 9, 4), np.float32)
        if kind != "zero":
            m[..., 0] = ((xx - 4) ** 2 + (yy - 6) ** 2 < 16) * (-1.0 if kind == "negative" else 1.0)
    sb.texture(m, aperture_mask=True)
    sb.texture(np.ones((4, 4, 4), np.float32))          # an unflagged texture next to it
    rc, rep = lg.scene_check(sb)
    assert rc == 0, rep
