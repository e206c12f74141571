"""Copies the reference's sample scene file (sample-scene-data/scene.json, written by the
reference's own exporter, Utils::exportScene) into tests/golden/reference_sample_scene.json, and
records the world-space spheres its scene graph flattens to under the oracle (oracle/scene_graph.py).

    python tests/golden/make_scene_fixtures.py <path to the reference tree>

The copied file is data the reference produced, not source: it pins both the reader (every key the
reference writes) and the writer (the library must write it back byte for byte)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import scene_graph as osg  # noqa: E402


def main() -> None:
    if len(sys.argv) != 2:
        sys.exit("usage: make_scene_fixtures.py <path to the reference tree>")
    ref = Path(sys.argv[1])
    text = (ref / "sample-scene-data" / "scene.json").read_bytes()
    (HERE / "reference_sample_scene.json").write_bytes(text)
    flat = osg.flatten_file_text(text.decode())
    out = {"source": "sample-scene-data/scene.json",
           "spheres": [[float(c) for c in s[:4]] + [int(s[4])] for s in flat]}
    (HERE / "reference_sample_scene_flat.json").write_text(json.dumps(out, indent=1) + "\n")
    print(out)


if __name__ == "__main__":
    main()
