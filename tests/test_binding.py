"""The GPU module's Lambda-side binding (lambda_gb300/binding) on lambda::Scene objects built by the
reference's own classes (oracle/ref_li.cpp), host only: each scene description becomes a
lambda::Scene, the binding translates it back (lambda_gpu::SceneDesc), and the translation must
compile to the same device scene as the original -- the report of lgpu_scene_check (BVH nodes and
depth, triangles, instances, shader-program length, light-tree nodes, distribution pool, tree power)
is compared whole.  The loader feeds some unlinked inputs through constant nodes of its own, so the
translation may have more nodes; they fold into the same programs."""
import pytest

from oracle import reference as R

pytestmark = pytest.mark.skipif(R.binding_lib() is None, reason=str(R.binding_unavailable_reason()))


def _scenes():
    from lambda_gb300 import abi, configs
    return {
        "cornell": lambda: configs.cornell(32, 32, 4),
        "node_zoo_power": lambda: configs.node_zoo(),
        "node_zoo_tree": lambda: configs.node_zoo(light_strategy=abi.LIGHT_STRATEGY_TREE),
        "volume_instances": lambda: configs.volume(32, 32, 1, n_instances=20, sphere_res=(24, 24)),
        "terrain": lambda: configs.terrain(32, 32, 1, grid=64, n_emitters=50),
        "cornell_inverse_textured": lambda: configs.cornell_inverse(32, 32, 4, tex_res=8),
    }


@pytest.mark.parametrize("name", list(_scenes()))
def test_binding_translation_compiles_to_the_same_scene(name):
    import lambda_gb300 as lg
    sb = _scenes()[name]()[0]
    b = R.BindingScene(sb)
    try:
        rc, report, counts = b.check()
    finally:
        b.close()
    assert rc == 0, report
    d = sb.desc()
    assert counts["meshes"] == d.num_meshes and counts["objects"] == d.num_objects
    assert counts["materials"] == d.num_materials and counts["lights"] == d.num_lights
    assert counts["media"] == d.num_media and counts["textures"] == d.num_textures
    assert counts["has_volumes"] == d.has_volumes and counts["light_strategy"] == d.light_strategy
    assert counts["nodes"] >= d.num_nodes
    rc0, report0 = lg.scene_check(sb)
    assert rc0 == 0 and report == report0, (report, report0)
