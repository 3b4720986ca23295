"""Host side of the headless renderer: camera matrices and fixed tables, against
independent numpy restatements of the same formulas."""
from __future__ import annotations

import math

import numpy as np

import nbody_gb300 as nb


def test_default_camera_matches_look_at_and_infinite_perspective():
    # Camera() defaults (camera.cpp:12-20): azimuth 0, elevation pi/4, distance 50.
    W, H = 1280, 720
    view, proj = nb.camera_matrices(0.0, math.pi / 4, 50.0, W, H)
    V = view.reshape(4, 4).T  # column-major -> row-major
    P = proj.reshape(4, 4).T
    eye = np.array([math.cos(0) * math.cos(math.pi / 4), math.sin(0) * math.cos(math.pi / 4),
                    math.sin(math.pi / 4)]) * 50.0
    f = -eye / np.linalg.norm(eye)
    s = np.cross(f, [0, 0, 1])
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    Vref = np.eye(4)
    Vref[0, :3], Vref[1, :3], Vref[2, :3] = s, u, -f
    Vref[:3, 3] = [-s @ eye, -u @ eye, f @ eye]
    assert np.allclose(V, Vref, atol=1e-5)
    t = math.tan(math.radians(30) / 2)
    Pref = np.zeros((4, 4))
    Pref[0, 0] = 1 / (t * W / H)
    Pref[1, 1] = 1 / t
    Pref[2, 2] = -1
    Pref[3, 2] = -1
    Pref[2, 3] = -2
    assert np.allclose(P, Pref, atol=1e-6)
    # the look-at point projects to the screen centre
    c = P @ V @ np.array([0, 0, 0, 1.0])
    assert abs(c[0] / c[3]) < 1e-6 and abs(c[1] / c[3]) < 1e-6


def test_render_tables_match_reference_formulas():
    off, w, flare = nb.render_tables()
    # gaussKernel(10, 25) (renderer_gl.cpp:314-336) + optimGaussKernel (:339-368)
    g = np.array([1 / (10 * math.sqrt(2 * math.pi)) * math.exp(-n * n / 200.0)
                  for n in range(25)])
    g /= 2 * g[1:].sum() + g[0]
    assert len(w) == 13 and abs(w[0] - g[0]) < 1e-7 and off[0] == 0
    for i in range(1, 13):
        ww = g[2 * i - 1] + g[2 * i]
        assert abs(w[i] - ww) < 1e-7
        assert abs(off[i] - ((2 * i - 1) * g[2 * i - 1] + 2 * i * g[2 * i]) / ww) < 1e-5
    assert abs(w[0] + 2 * w[1:].sum() - 1.0) < 1e-6   # normalised
    # genFlareTex(16) (gen.cpp:36-51): gamma-corrected Gaussian, sigma^2 = 8
    i1 = np.arange(16) - 8
    ref = np.exp(-(i1[:, None] ** 2 / 16.0 + i1[None, :] ** 2 / 16.0)) ** 2.2
    assert np.allclose(flare, ref, rtol=1e-5, atol=1e-7)
    assert flare[8, 8] == 1.0
