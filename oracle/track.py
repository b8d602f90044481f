"""TEST INFRASTRUCTURE ONLY: numpy restatements of the reference's tracking
loop helpers (TW/TW_Core/cuda_utils.cu:109-240, fftcctworkerthread.cpp:228-330):
the reference-refresh POI update and the fixed-range displacement colour map."""
import numpy as np


def jet256() -> np.ndarray:
    """The 256-entry colour map as RGBA uint32 (red lowest byte): piecewise
    linear ramps of a(k) = round(255 k / 64), blue -> cyan -> yellow -> red
    (the reference's texture_data, TW/TW_Core/cuda_utils.cu:15-47)."""
    a = lambda k: (255 * k + 32) // 64  # noqa: E731
    out = np.zeros(256, np.uint32)
    for i in range(256):
        if i < 32:
            r, g, b = 0, 0, a(i + 33)
        elif i < 96:
            r, g, b = 0, a(i - 31), 255
        elif i < 160:
            r, g, b = a(i - 95), 255, a(159 - i)
        elif i < 224:
            r, g, b = 255, a(223 - i), 0
        else:
            r, g, b = a(287 - i), 0, 0
        out[i] = 0xFF000000 | (b << 16) | (g << 8) | r
    return out


def track_update(poi, u, v, acc_u, acc_v, lo_y, hi_y, lo_x, hi_x):
    """accumulateUV then updatePOIpos (cuda_utils.cu:174-240): acc += (u, v);
    (y, x) += (int(v), int(u)), held in [lo, hi]."""
    acc_u = (acc_u + u).astype(np.float32)
    acc_v = (acc_v + v).astype(np.float32)
    p = poi.copy()
    p[:, 0] = np.clip(p[:, 0] + np.trunc(v).astype(np.int32), lo_y, hi_y)
    p[:, 1] = np.clip(p[:, 1] + np.trunc(u).astype(np.int32), lo_x, hi_x)
    return p, acc_u, acc_v


def colormap(tex_u, tex_v, poi, u, v, acc_u, acc_v, sx, sy, rw, rh, min_u, max_u, min_v, max_v):
    """constructTextImageFixedMinMax (cuda_utils.cu:109-172) at the displayed
    positions of accumulatePOI; float32 arithmetic as the kernel's."""
    jet = jet256()
    f32 = np.float32

    def color(t, lo, hi):
        t = np.minimum(t, f32(hi))
        t = np.maximum(t, f32(lo))
        t = (t - f32(lo)).astype(f32)
        k = np.trunc((f32(255.0) * t).astype(f32) / f32(f32(hi) - f32(lo))).astype(np.int64)
        return jet[np.clip(k, 0, 255)]

    cu = color((u + acc_u).astype(f32), min_u, max_u)
    cv = color((v + acc_v).astype(f32), min_v, max_v)
    ys = poi[:, 0] + np.trunc(v).astype(np.int64) - sy
    xs = poi[:, 1] + np.trunc(u).astype(np.int64) - sx
    tex_u, tex_v = tex_u.copy(), tex_v.copy()
    for i in range(len(poi)):  # later POIs overwrite earlier ones where blocks overlap
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                yy, xx = ys[i] + dy, xs[i] + dx
                if 0 <= yy < rh and 0 <= xx < rw:
                    tex_u[yy, xx] = cu[i]
                    tex_v[yy, xx] = cv[i]
    return tex_u, tex_v
