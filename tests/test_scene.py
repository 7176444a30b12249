"""CPU: the synthetic scene generator (host path) is deterministic and matches the
workload description (depth range, sky, roughness, candidate formats)."""
import numpy as np

import violet_gb300 as vg


def test_deterministic_and_seeded():
    a = vg.Scene(3, 96, 64).generate_host(2)
    b = vg.Scene(3, 96, 64).generate_host(2)
    c = vg.Scene(4, 96, 64).generate_host(2)
    for k in a:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert not np.array_equal(a["depth"], c["depth"])


def test_workload_statistics():
    W, H = 320, 180
    s = vg.Scene(11, W, H, disocclusion_frac=0.02)
    f = s.generate_host(1)
    d = f["depth"]
    geo = d > 0
    assert 0.6 < geo.mean() < 1.0
    # reverse-Z with near 0.05: depth ~ 0.05 / z; geometry within 50 m
    z = 0.05 / d[geo]
    assert z.max() < 55 and z.min() > 0.5
    g1 = f["gbuffer"][W * H: 2 * W * H]
    rough = (g1 >> 24)[geo] / 255.0
    assert rough.min() < 0.1 and rough.max() > 0.95
    assert np.all(f["gbuffer"][3 * W * H:][geo] == 1) and np.all(f["gbuffer"][3 * W * H:][~geo] == 0)
    assert np.all(f["spec_hit_pos"].reshape(-1, 4)[geo, 3] == 1.0)
    pdf = f["diff_source_pdf"][geo]
    assert np.all(pdf >= 0) and np.all(pdf <= 1 / np.pi + 1e-6)


def test_frame_params_camera_motion_and_jitter():
    s = vg.Scene(1, 320, 180)
    p0, p1 = s.frame_params(0), s.frame_params(1)
    v0 = np.array(p0.view_pos[:3])
    v1 = np.array(p1.view_pos[:3])
    assert abs(np.linalg.norm(v1 - v0) - 0.01) < 1e-6
    assert np.allclose(np.array(p1.prev_view_pos[:3]), v0)
    assert p0.jitter[2] == 0 and p0.jitter[3] == 0
    assert np.isclose(p1.jitter[2], p0.jitter[0]) and np.isclose(p1.jitter[3], p0.jitter[1])
    vp = np.array(p0.view_proj).reshape(4, 4).T
    ivp = np.array(p0.inv_view_proj).reshape(4, 4).T
    assert np.allclose(vp @ ivp, np.eye(4), atol=1e-4)
    # Halton(2,3) jitter of index 1 (render_loop.rs:89-95): (2*0.5-1, 2*(1/3)-1) / size
    assert np.isclose(p0.jitter[0], 0.0) and np.isclose(p0.jitter[1], (2 / 3 - 1) / 180)


def _halton(i, b):
    f, r = 1.0, 0.0
    while i > 0:
        f /= b
        r += f * (i % b)
        i //= b
    return r


def test_jitter_is_the_halton_2_3_cycle_of_eight():
    # render_loop.rs:89-106 with the cycle of restir_renderer.rs:65: frame f jitters by
    # Halton(2, 3) of index f % 8 + 1, mapped to [-1, 1) and divided by the size.
    W, H = 320, 180
    s = vg.Scene(1, W, H)
    for f in range(17):
        p = s.frame_params(f)
        k = f % 8 + 1
        assert np.isclose(p.jitter[0], (2 * _halton(k, 2) - 1) / W, atol=1e-9), f
        assert np.isclose(p.jitter[1], (2 * _halton(k, 3) - 1) / H, atol=1e-9), f


def test_reverse_z_projection():
    # perspective_projection of app.rs:28-56 with near 0.05, far 102400: a point at
    # view depth t on the principal axis (NDC x, y = the frame's jitter) has NDC depth
    # m22 + m23 / t, 1 at the near plane and 0 at the far plane.
    near, far = 0.05, 102400.0
    m22, m23 = -near / (far - near), near / (1.0 - near / far)
    s = vg.Scene(3, 320, 180)
    p = s.frame_params(0)
    ivp = np.array(p.inv_view_proj, np.float64).reshape(4, 4).T
    cam = np.array(p.view_pos[:3], np.float64)
    for t in (0.05, 0.5, 5.0, 50.0):
        ndc = np.array([p.jitter[0], p.jitter[1], m22 + m23 / t, 1.0])
        w = ivp @ ndc
        assert np.isclose(np.linalg.norm(w[:3] / w[3] - cam), t, rtol=2e-5), t


def test_host_only_generator_matches_the_product_library():
    """The oracle's copy of the scene generator (the product's source compiled without
    CUDA, used by the CPU benchmark) produces the same frames as the product library."""
    from oracle import pyscene

    W, H = 96, 54
    a = vg.Scene(1000, W, H, disocclusion_frac=0.02)
    b = pyscene.Scene(1000, W, H, disocclusion_frac=0.02)
    for f in (0, 5):
        assert bytes(a.frame_params(f)) == bytes(b.frame_params(f))
        ha, hb = a.generate_host(f), b.generate_host(f)
        assert ha.keys() == hb.keys()
        for k in ha:
            assert np.array_equal(ha[k].view(np.uint8), hb[k].view(np.uint8)), k


def test_benchmark_knobs_are_the_plain_1080p_preset():
    import bench

    p = vg.params_plain(1)
    assert {k: getattr(p, k) for k, _ in p._fields_} == bench.WORKLOAD_KNOBS
