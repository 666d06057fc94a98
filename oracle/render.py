"""CPU restatement of the headless particle image (lennard-jones-cuda_gb300/
csrc/lj_render.cu), operation for operation in FP64 with separately rounded
operations, for exact comparison (test infrastructure only).  The image
stands in for the reference's OpenGL viewer (src/gui/MDSystemGL.cpp:32-160):
orange (255, 127, 0) spheres of radius 0.5 sigma."""
from __future__ import annotations

import numpy as np


def _orderable(f32):
    b = np.float32(f32).view(np.uint32)
    return int(~b & 0xffffffff) if b & 0x80000000 else int(b | 0x80000000)


def render(pos, L, axis, W, H, R):
    ca = 1 if axis == 0 else 0
    cb = 1 if axis == 2 else 2
    key = np.zeros(W * H, dtype=object)
    key[:] = 0
    sx, sy = L / W, L / H
    R2 = R * R
    for k, p in enumerate(np.asarray(pos, np.float64)):
        u, v = p[ca] / sx, p[cb] / sy
        depth = p[axis]
        i0 = max(0, int(np.floor(u - R / sx)) - 1)
        i1 = min(W - 1, int(np.floor(u + R / sx)) + 1)
        j0 = max(0, int(np.floor(v - R / sy)) - 1)
        j1 = min(H - 1, int(np.floor(v + R / sy)) + 1)
        for j in range(j0, j1 + 1):
            dy = ((j + 0.5) - v) * sy
            dy2 = dy * dy
            for i in range(i0, i1 + 1):
                dx = ((i + 0.5) - u) * sx
                d2 = dx * dx + dy2
                if not d2 < R2:
                    continue
                surf = depth + np.sqrt(R2 - d2)
                kk = (_orderable(np.float32(surf)) << 32) | (k + 1)
                if kk > key[j * W + i]:
                    key[j * W + i] = kk
    img = np.zeros((H, W, 4), np.uint8)
    img[:, :, 3] = 255
    for pix in range(W * H):
        kk = key[pix]
        if not kk:
            continue
        i, j = pix % W, pix // W
        k = (kk & 0xffffffff) - 1
        p = pos[k]
        u, v = p[ca] / sx, p[cb] / sy
        dx = ((i + 0.5) - u) * sx
        dy = ((j + 0.5) - v) * sy
        d2 = dx * dx + dy * dy
        nz = np.sqrt(1.0 - d2 / (R * R))
        f = 0.3 + 0.7 * nz
        for c, col in enumerate((255.0, 127.0, 0.0)):
            img[H - 1 - j, i, c] = int(np.floor(col * f + 0.5))
    return img
