"""Scene files and scene-graph flattening (atx_scene_*) against the oracle's restatement of
Utils.cpp:97-187, SceneNode.cpp:42-59 and Renderer.cu:25-37, 67-96, and against the reference's own
sample scene file (written by its exporter)."""
import json
import struct
from pathlib import Path

import numpy as np
import pytest

import ataraxia_gb300 as atx
from ataraxia_gb300 import _native as N
from oracle import scene_graph as osg

GOLDEN = Path(__file__).resolve().parent / "golden"
SAMPLE = GOLDEN / "reference_sample_scene.json"


def bits(x) -> int:
    return struct.unpack("<I", struct.pack("<f", float(x)))[0]


def random_scene(seed: int, depth: int = 4, fanout: int = 3, n_mat: int = 5, unit_quat: bool = True) -> dict:
    rng = np.random.default_rng(seed)

    def node(name, d):
        q = rng.normal(size=4)
        if unit_quat:
            q /= np.linalg.norm(q)
        n = {"name": name,
             "transformation": {"position": rng.uniform(-10, 10, 3).tolist(), "rotation": q.tolist(),
                                "scale": rng.uniform(0.2, 3.0, 3).tolist()}}
        ns = int(rng.integers(0, 4))
        if ns:
            n["spheres"] = [{"center": rng.uniform(-5, 5, 3).tolist(), "radius": float(rng.uniform(0.1, 2)),
                             "materialIndex": int(rng.integers(-2, n_mat + 2))} for _ in range(ns)]
        if d < depth:
            kids = [node(f"{name}.{k}", d + 1) for k in range(int(rng.integers(0, fanout + 1)))]
            if kids:
                n["children"] = kids
        return n

    mats = [{"albedo": rng.uniform(0, 1, 3).tolist(), "roughness": float(rng.uniform()),
             "metallic": float(rng.integers(0, 2)), "F0": [0.04] * 3, "emissionIntensity": 0.0,
             "emissionColor": [0.0, 0.0, 0.0]} for _ in range(n_mat)]
    return {"camera": {"position": [0.0, 2.0, 10.0], "direction": [0.0, -0.2, -1.0], "fov": 45.0},
            "sceneGraph": node("Scene", 0), "materials": mats,
            "lights": [{"position": [0.0, 8.0, 0.0], "intensity": 50.0, "color": [1.0, 1.0, 1.0]}],
            "settings": {"maxBounces": 5, "skyLight": False, "accumulation": True}}


# ------------------------------------------------------------- sample scene

def test_reference_sample_scene_imports_and_flattens():
    sc = atx.import_scene(SAMPLE)
    flat = json.loads((GOLDEN / "reference_sample_scene_flat.json").read_text())["spheres"]
    s = sc.arrays()[0]
    assert len(s) == len(flat) == 3
    for got, want in zip(s, flat):
        assert [bits(v) for v in list(got["center"]) + [got["radius"]]] == [bits(v) for v in want[:4]]
        assert int(got["material"]) == want[4]
    info = sc.graph.info()
    assert info["n_nodes"] == 3 and info["n_materials"] == 3 and info["n_lights"] == 1
    assert sc.settings == atx.Settings(accumulation=True, skyLight=False, maxBounces=25)
    assert sc.camera.fov == 45.0 and (sc.camera.nearClip, sc.camera.farClip) == (np.float32(0.1), 100.0)
    j = json.loads(SAMPLE.read_text())
    assert [bits(v) for v in sc.camera.position] == [bits(v) for v in j["camera"]["position"]]
    m = sc.materials
    assert [bits(v) for v in m["albedo"][0]] == [bits(v) for v in j["materials"][0]["albedo"]]


def test_reference_sample_scene_writes_back_byte_for_byte():
    text = SAMPLE.read_text()
    g = atx.SceneGraph.from_json(text)
    assert g.to_json() == text


def test_save_and_load_file(tmp_path):
    sc = atx.import_scene(SAMPLE)
    p = tmp_path / "scene.json"
    atx.export_scene(sc, p)
    assert p.read_text() == SAMPLE.read_text()
    with pytest.raises(atx.AtxError) as e:
        atx.import_scene(tmp_path / "missing.json")
    assert e.value.status == 6          # ATX_ERR_NOT_FOUND


# --------------------------------------------------------- random graphs

@pytest.mark.parametrize("seed", range(12))
def test_flatten_bit_exact_vs_oracle(seed):
    j = random_scene(seed, unit_quat=seed % 3 != 0)
    text = json.dumps(j)
    got = atx.SceneGraph.from_json(text).flatten()
    want = osg.flatten(j["sceneGraph"], len(j["materials"]))
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert [bits(v) for v in list(g["center"]) + [g["radius"]]] == [bits(v) for v in w[:4]]
        assert int(g["material"]) == w[4]


@pytest.mark.parametrize("seed", range(4))
def test_flatten_close_to_float64(seed):
    j = random_scene(100 + seed)
    got = atx.SceneGraph.from_json(json.dumps(j)).flatten()
    want = osg.flatten_f64(j["sceneGraph"], len(j["materials"]))
    g = np.array([list(s["center"]) + [s["radius"]] for s in got], dtype=np.float64)
    w = np.array([x[:4] for x in want], dtype=np.float64)
    # float32 through up to five nested transforms with |t| <= 10
    np.testing.assert_allclose(g, w, rtol=1e-4, atol=2e-4)


def test_material_index_clamped():
    j = random_scene(7, n_mat=2)
    got = atx.SceneGraph.from_json(json.dumps(j)).flatten()
    assert ((got["material"] >= 0) & (got["material"] < 2)).all()


def test_json_round_trip_is_stable():
    j = random_scene(3)
    g1 = atx.SceneGraph.from_json(json.dumps(j))
    t1 = g1.to_json()
    g2 = atx.SceneGraph.from_json(t1)
    assert g2.to_json() == t1
    assert g1.flatten().tobytes() == g2.flatten().tobytes()
    # the text is plain JSON carrying the same values (as float32)
    back = json.loads(t1)
    assert back["sceneGraph"]["name"] == "Scene"
    assert [bits(v) for v in back["materials"][1]["albedo"]] == [bits(v) for v in j["materials"][1]["albedo"]]
    assert list(back.keys()) == sorted(back.keys())


def test_number_format():
    g = atx.SceneGraph()
    lt = np.zeros(1, dtype=atx.LIGHT_DTYPE)
    vals = [1e-5, 1e20, 0.1, 123456789.0, 0.001, 2.5, 1e15, 1e16]
    lt[0]["position"] = vals[:3]
    lt[0]["color"] = vals[3:6]
    lt[0]["intensity"] = vals[6]
    g.set_lights(lt)
    t = g.to_json()
    light = json.loads(t)["lights"][0]
    for got, want in zip(light["position"] + light["color"] + [light["intensity"]], vals):
        assert bits(got) == bits(want)
    # json::dump layout of floats widened to double: fixed notation for decimal exponents in
    # (-4, 15], otherwise d.ddde[+-]XX with two exponent digits at least
    assert '"intensity": 999999986991104.0' in t
    assert "9.999999747378752e-06" in t and "1.0000000200408773e+20" in t
    assert "0.10000000149011612" in t and "123456792.0" in t and "2.5" in t


def test_edit_api_matches_file():
    g = atx.SceneGraph()
    s = np.zeros(1, dtype=atx.SPHERE_DTYPE)
    s[0] = ((0.0, 0.0, 0.0), 1.0, 0)
    g.add_spheres(atx.ROOT, s)
    c = g.add_node(atx.ROOT, "ChildNode1")
    g.set_transform(c, position=(2, 0, 0), rotation_xyzw=(0, 0, 0, 0), scale=(1, 1, 1))
    s[0] = ((0.0, -101.0, 0.0), 100.0, 1)
    g.add_spheres(c, s)
    gc = g.add_node(c, "GrandChildNode")
    g.set_transform(gc, position=(0, 0, 0), rotation_xyzw=(0, 0, 0, 0), scale=(1, 1, 1))
    s[0] = ((1.0, 0.0, 0.0), 1.0, 2)
    g.add_spheres(gc, s)
    ref = atx.SceneGraph.from_json(SAMPLE.read_text())
    g.set_materials(ref.materials())
    g.set_lights(ref.lights())
    i = ref.info()
    cam = N.CameraDesc()
    cam.position[:] = i["camera"]["position"]
    cam.direction[:] = i["camera"]["direction"]
    cam.fov_deg, cam.near_clip, cam.far_clip = i["camera"]["fov"], 0.1, 100.0
    g.set_camera(cam)
    g.set_settings(N.Settings(1, 0, (0, 0), 25))
    assert g.to_json() == SAMPLE.read_text()
    assert g.flatten().tobytes() == ref.flatten().tobytes()


# ----------------------------------------------------------------- errors

@pytest.mark.parametrize("text,needle", [
    ("", "unexpected end"),
    ('{"camera": {"position": [0, 0, 0], "direction": [0, 0, -1], "fov": 45}', "expected ',' or '}'"),
    ('{"settings": {"maxBounces": 5, "skyLight": false, "accumulation": true}}', "camera"),
    ('{"camera": {"position": [0, 0], "direction": [0, 0, -1], "fov": 45}, '
     '"settings": {"maxBounces": 5, "skyLight": false, "accumulation": true}}', "position"),
    ('{"camera": {"position": [0, 0, 0], "direction": [0, 0, -1], "fov": "wide"}, '
     '"settings": {"maxBounces": 5, "skyLight": false, "accumulation": true}}', "fov"),
    ('{"camera": {"position": [0, 0, 0], "direction": [0, 0, -1], "fov": 45}, '
     '"settings": {"maxBounces": 5, "skyLight": 0, "accumulation": true}}', "skyLight"),
    ('[' * 400 + ']' * 400, "nesting too deep"),
    ('{"a": tru}', "invalid literal"),
    ('{"a": 01}', "expected ',' or '}'"),
    ('{"a": "\\x"}', "invalid escape"),
    ('{"a": 1} x', "trailing characters"),
])
def test_parse_errors(text, needle):
    with pytest.raises(atx.AtxError) as e:
        atx.SceneGraph.from_json(text)
    assert e.value.status == 9          # ATX_ERR_PARSE
    assert needle in e.value.message


def test_error_position_reported():
    with pytest.raises(atx.AtxError) as e:
        atx.SceneGraph.from_json('{\n  "camera": {\n    "fov": 45,,\n')
    assert "line 3" in e.value.message


def test_unicode_names_round_trip():
    g = atx.SceneGraph()
    g.add_node(atx.ROOT, 'né中"\\\n\x01')
    back = json.loads(g.to_json())
    assert back["sceneGraph"]["children"][0]["name"] == 'né中"\\\n\x01'
    g2 = atx.SceneGraph.from_json(json.dumps(back))
    assert g2.to_json() == g.to_json()


def test_deep_graph_bounded():
    g = atx.SceneGraph()
    k = atx.ROOT
    for _ in range(256):
        k = g.add_node(k, "n")
    with pytest.raises(atx.AtxError):
        g.add_node(k, "too deep")


# ------------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_sample_scene_renders_as_the_oracle():
    """The reference's own scene file through the renderer, bit-exact against the oracle."""
    from oracle import pyoracle as po

    sc = atx.import_scene(SAMPLE)
    spheres, mats, lights = sc.arrays()
    w, h, spp = 48, 27, 3
    cam = sc.camera
    po.build()
    _, iv, _, ip = po.camera_matrices(cam.position, cam.direction, cam.fov, cam.nearClip, cam.farClip, w, h)
    view = po.make_view(iv, ip, cam.position, w, h)
    acc_o, _, _ = po.render(spheres, mats, lights, view, max_bounces=sc.settings.maxBounces, spp=spp, mode=po.EXACT)
    with atx.Renderer() as r:
        r.on_resize(w, h)
        r.set_scene_graph(sc.graph)
        r.set_camera_matrices(np.array(view.inv_view), np.array(view.inv_proj), cam.position)
        r.set_settings(sc.settings)
        r.render_frames(spp)
        acc = r.get_accumulation().reshape(-1, 4)
    assert np.array_equal(acc.view(np.uint32), np.asarray(acc_o, dtype=np.float32).reshape(-1, 4).view(np.uint32))
