"""The restated reference kernel (baseline/refport, a bench measuring stick) computes the same
estimator: built with the reference's fast-math flags its frames differ from the oracle's only at
rounding level, so image means agree closely."""
import numpy as np
import pytest

from ataraxia_gb300 import Camera, camera_matrices, scenes
from tests.helpers import frac_outside, oracle_render

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["config0", "config1"])
def test_refport_matches_oracle_statistically(po, name):
    from baseline import refport

    sc = {"config0": scenes.config0, "config1": scenes.config1}[name]().with_resolution(160, 90)
    cam = Camera(sc.fov, sc.near, sc.far, sc.camera_position, sc.camera_direction)
    _, iv, _, ip = camera_matrices(cam, sc.width, sc.height)
    port = refport.RefPort(sc.spheres, sc.materials, sc.lights, sc.width, sc.height,
                           refport.ray_dirs(iv, ip, sc.width, sc.height), sc.camera_position, sc.max_bounces)
    try:
        for _ in range(8):
            port.frame()
        acc = port.accumulation()
    finally:
        port.close()
    lit, _, _ = oracle_render(sc, 8, mode=po.LITERAL)
    assert np.all(acc[:, 3] == 8.0)
    m_port, m_ref = acc[:, :3].mean(), lit[:, :3].mean()
    assert abs(m_port - m_ref) <= 0.02 * abs(m_ref) + 1e-4, (m_port, m_ref)
    print(f"{name}: refport vs literal oracle, pixels outside 1e-3: {frac_outside(acc, lit):.3%}")
