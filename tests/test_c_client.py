"""The C ABI from C: include/atx.h compiles as C99 with warnings as errors, a client links against
libatx.so, and on a GPU it renders the reference's sample scene to the same image as the Python
binding."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "c_client" / "render_scene.c"
SAMPLE = ROOT / "tests" / "golden" / "reference_sample_scene.json"


def build_client(tmp_path, native):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lib = ROOT / "ataraxia_gb300" / "_lib"
    exe = tmp_path / "render_scene"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(SRC),
                    "-L", str(lib), "-latx", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return exe


def test_header_compiles_as_c_and_client_links(tmp_path, native):
    exe = build_client(tmp_path, native)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 2 and "usage" in out.stderr


def test_bad_scene_file_reports_error(tmp_path, native):
    exe = build_client(tmp_path, native)
    bad = tmp_path / "bad.json"
    bad.write_text('{"camera": {')
    out = subprocess.run([str(exe), str(bad), str(tmp_path / "x.ppm"), "8", "8", "1"], capture_output=True,
                         text=True)
    assert out.returncode == 1 and "parse error" in out.stderr and "line" in out.stderr


@pytest.mark.gpu
def test_c_client_renders_like_python(tmp_path, native):
    import ataraxia_gb300 as atx

    exe = build_client(tmp_path, native)
    out = subprocess.run([str(exe), str(SAMPLE), str(tmp_path / "c.ppm"), "160", "90", "8"], capture_output=True,
                         text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith("frame 9 ")
    sc = atx.import_scene(SAMPLE)
    with atx.Renderer() as r:
        r.on_resize(160, 90)
        r.set_scene_graph(sc.graph)
        r.set_settings(sc.settings)
        r.set_camera(sc.camera)
        r.render_frames(8)
        r.save_image(tmp_path / "py.ppm")
    assert (tmp_path / "c.ppm").read_bytes() == (tmp_path / "py.ppm").read_bytes()
