"""CPU restatement of the headless point splat (gi_splat.cu).

TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/ import this module.
The camera follows gluLookAt + glFrustum as the reference's viewer sets them
up (impactAddTime.cu:535-538); every operation is a float32 numpy operation
in the kernel's order, so the image is reproduced exactly.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32

# Colours of commonSetup.h:125-128 as 8-bit RGB: Fe body 1, Fe body 2,
# Si body 1, Si body 2; then the analysis picture's Earth and Moon
# (impactBasicFunctions.h:758-771).
RGB = [(255, 255, 0), (255, 0, 0), (99, 66, 33), (181, 102, 28)]
RGB_SCOPE = [(0, 0, 255), (255, 255, 255)]


def splat(pos, bounds, basis, near, far, half, width, height, point_size, scope=None):
    """bounds colour by origin and material; with scope (n bytes) only
    scope 1 (Earth) and 2 (Moon) elements are drawn, in their colours."""
    b = np.asarray(basis, dtype=np.float32)
    s, u, f, eye = b[0:3], b[3:6], b[6:9], b[9:12]
    p = np.asarray(pos, dtype=np.float32)[:, :3]
    d = p - eye

    def dot(a):
        return (a[0] * d[:, 0] + a[1] * d[:, 1]) + a[2] * d[:, 2]

    depth = dot(f)
    xe, ye = dot(s), dot(u)
    k = f32(near) / f32(half)
    with np.errstate(divide="ignore", invalid="ignore"):
        xn = (k * xe) / depth
        yn = (k * ye) / depth
    ok = (depth >= f32(near)) & (depth <= f32(far)) & (np.abs(xn) <= 2) & (np.abs(yn) <= 2)
    if scope is not None:
        sc = np.asarray(scope)
        ok &= (sc == 1) | (sc == 2)
    idx = np.flatnonzero(ok)
    wx = (xn[idx] + f32(1)) * f32(0.5 * width)
    wy = (f32(1) - yn[idx]) * f32(0.5 * height)
    lo = f32(0.5 * point_size - 0.5)
    x0 = np.floor(wx - lo).astype(np.int64)
    y0 = np.floor(wy - lo).astype(np.int64)
    if scope is None:
        cls = np.where(idx < bounds[0], 0, np.where(idx < bounds[1], 1, np.where(idx < bounds[2], 2, 3)))
    else:
        cls = 3 + np.asarray(scope)[idx].astype(np.int64)
    rgb = np.array([(r << 16) | (g << 8) | bb for r, g, bb in RGB + RGB_SCOPE], np.uint64)[cls]
    key = (depth[idx].view(np.uint32).astype(np.uint64) << np.uint64(32)) | rgb
    z = np.full(width * height, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    for dy in range(point_size):
        for dx in range(point_size):
            xx, yy = x0 + dx, y0 + dy
            m = (xx >= 0) & (xx < width) & (yy >= 0) & (yy < height)
            np.minimum.at(z, (yy[m] * width + xx[m]), key[m])
    c = np.where(z == np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64(0), z & np.uint64(0xFFFFFF))
    img = np.zeros((height * width, 3), np.uint8)
    img[:, 0] = (c >> np.uint64(16)).astype(np.uint8)
    img[:, 1] = ((c >> np.uint64(8)) & np.uint64(255)).astype(np.uint8)
    img[:, 2] = (c & np.uint64(255)).astype(np.uint8)
    return img.reshape(height, width, 3)
