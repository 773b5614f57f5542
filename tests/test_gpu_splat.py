"""GPU tests of the headless point splat (gi_splat) against its CPU
restatement, pixel for pixel, and of frame playback to PPM files."""
from __future__ import annotations

import numpy as np
import pytest

import splat_oracle as so

pytestmark = pytest.mark.gpu


def _scene(seed, n):
    rng = np.random.default_rng(seed)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.normal(scale=12.0, size=(n, 3))
    pos[: n // 10, :3] = pos[n // 10: 2 * (n // 10), :3]  # coincident pairs: depth ties
    return pos


@pytest.mark.parametrize("point_size,eye", [(2, (0.0, 0.0, 80.0)), (3, (55.0, -30.0, 40.0)),
                                            (1, (0.0, 0.0, 5.0))])
def test_splat_matches_restatement(gi, torch_cuda, point_size, eye):
    torch = torch_cuda
    n = 20000
    pos = _scene(1, n)
    bounds = [2000, 4000, 12000]
    v = gi.view(eye, up=(0.0, 1.0, 0.0), width=320, height=240, point_size=point_size)
    ctx = gi.Context(0)
    d = torch.from_numpy(pos).cuda()
    img = gi.splat(ctx, d.data_ptr(), n, bounds, v)
    want = so.splat(pos, bounds, gi.view_basis(v), v.near_plane, v.far_plane, v.frustum_half,
                    v.width, v.height, v.point_size)
    assert np.array_equal(img, want)
    assert (img.sum(2) > 0).mean() > 0.01  # something was drawn
    colours = {tuple(c) for c in img.reshape(-1, 3)}
    assert {tuple(c) for c in so.RGB} & colours
    ctx.close()


def test_splat_rejects_bad_views(gi, torch_cuda):
    torch = torch_cuda
    ctx = gi.Context(0)
    d = torch.zeros((4, 4), device="cuda")
    for bad in (dict(width=0), dict(point_size=0), dict(near=-1.0), dict(far=0.1)):
        kw = dict(width=16, height=16, point_size=2, near=0.2, far=100.0)
        kw.update(bad)
        with pytest.raises(gi.GIError):
            gi.splat(ctx, d.data_ptr(), 4, [0, 0, 0], gi.view((0, 0, 10), **kw))
    with pytest.raises(gi.GIError):  # eye == center
        gi.splat(ctx, d.data_ptr(), 4, [0, 0, 0], gi.view((0, 0, 0), width=8, height=8))
    ctx.close()


def test_render_frames_to_ppm(gi, torch_cuda, tmp_path):
    torch = torch_cuda
    n = 3000
    b = gi.BodyParams(1, 1, 1, 2.5, 1.0, 1.0, 1, 1, 0.01, 0.01, 0.01, 0.01, n, 300, 1700, 100, 900)
    info = tmp_path / "info"
    info.mkdir()
    gi.write_body_params(str(info / "targetImpactorParameters"), b)
    frames = str(tmp_path / "impactPosVel")
    rng = np.random.default_rng(2)
    poses = []
    for k in range(5):
        pos = _scene(10 + k, n)
        poses.append(pos)
        gi.frames_append(frames, 0.1 * k, pos, np.zeros_like(pos))
    v = gi.view((0.0, 0.0, 60.0), width=64, height=48)
    wrote = gi.render_frames(str(info), frames, v, str(tmp_path / "img"), every=2)
    assert wrote == 3
    ctx = gi.Context(0)
    bounds = [300, 400, 2100]
    for k in (0, 2, 4):
        raw = open(tmp_path / f"img{k:05d}.ppm", "rb").read()
        head = b"P6\n64 48\n255\n"
        assert raw.startswith(head) and len(raw) == len(head) + 64 * 48 * 3
        d = torch.from_numpy(poses[k]).cuda()
        img = gi.splat(ctx, d.data_ptr(), n, bounds, v)
        assert raw[len(head):] == img.tobytes()
    ctx.close()


def test_analysis_splat_matches_restatement(gi, torch_cuda):
    """gi_splat_scope draws only Earth (scope 1, blue) and Moon (scope 2,
    white) elements, pixel for pixel as the restatement; fed by the GPU
    grouping, the two largest clumps come out blue and white."""
    torch = torch_cuda
    n = 20000
    pos = _scene(2, n)
    scope = np.random.default_rng(5).integers(0, 4, size=n).astype(np.uint8)
    v = gi.view((30.0, 20.0, 70.0), up=(0.0, 1.0, 0.0), width=320, height=240, point_size=2)
    ctx = gi.Context(0)
    d, ds = torch.from_numpy(pos).cuda(), torch.from_numpy(scope).cuda()
    img = gi.splat_scope(ctx, d.data_ptr(), n, ds.data_ptr(), v)
    want = so.splat(pos, None, gi.view_basis(v), v.near_plane, v.far_plane, v.frustum_half,
                    v.width, v.height, v.point_size, scope=scope)
    assert np.array_equal(img, want)
    colours = {tuple(c) for c in img.reshape(-1, 3)}
    assert colours <= {(0, 0, 0), (0, 0, 255), (255, 255, 255)}
    assert {(0, 0, 255), (255, 255, 255)} <= colours

    from test_groups_cpu import clumps
    cp = clumps(3, [900, 300, 40], spacing=1.2, far=25.0)
    m = len(cp)
    dc = torch.from_numpy(cp).cuda()
    sc = torch.zeros(m, dtype=torch.uint8, device="cuda")
    group = torch.zeros(m, dtype=torch.int32, device="cuda")
    em = gi.find_earth_moon(ctx, dc.data_ptr(), m, 1.5, [m // 5, 2 * m // 5, 3 * m // 5],
                            group.data_ptr(), sc.data_ptr())
    assert em.n_earth == 900 and em.n_moon == 300
    v2 = gi.view((25.0, 5.0, 120.0), center=(25.0, 5.0, 0.0), up=(0.0, 1.0, 0.0), width=320,
                 height=240, point_size=2)
    img2 = gi.splat_scope(ctx, dc.data_ptr(), m, sc.data_ptr(), v2)
    want2 = so.splat(cp, None, gi.view_basis(v2), v2.near_plane, v2.far_plane, v2.frustum_half,
                     v2.width, v2.height, v2.point_size, scope=sc.cpu().numpy())
    assert np.array_equal(img2, want2)
    c2 = {tuple(c) for c in img2.reshape(-1, 3)}
    assert {(0, 0, 255), (255, 255, 255)} <= c2
    ctx.close()
