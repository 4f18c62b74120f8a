"""Shared helpers for the GPU parity tests."""
import numpy as np


def planar_to_interleaved(a):
    """(3, rows, cols) -> (rows*cols, 3)"""
    return np.ascontiguousarray(np.moveaxis(a, 0, -1).reshape(-1, 3), dtype=np.float64)


def gpu_compose(pg, K, S, V, R0, storage="f32", fused=True, inplace=False):
    """K, S: (L, 3, rows, cols); V: (L, rows, cols); R0: (3, rows, cols) -> (3, rows, cols)."""
    L = V.shape[0]
    rows, cols = R0.shape[1:]
    layers = []
    for l in range(L):
        ly = pg.PaintLayer(rows, cols, storage)
        ly.upload("K", K[l], planar=True)
        ly.upload("S", S[l], planar=True)
        ly.upload("V", V[l], planar=True)
        layers.append(ly)
    img_storage = "f64" if storage == "f64" else "f32"
    r0 = pg.Image(rows, cols, img_storage)
    r0.upload(R0, planar=True)
    out = r0 if inplace else pg.Image(rows, cols, img_storage)
    pg.compose_layers(layers, r0, out, fused=fused)
    return out.download(dtype=np.float64, planar=True)


def oracle_compose(oracle, K, S, V, R0, mode=0):
    L = V.shape[0]
    Ko = np.stack([planar_to_interleaved(K[l]) for l in range(L)])
    So = np.stack([planar_to_interleaved(S[l]) for l in range(L)])
    Vo = V.reshape(L, -1).astype(np.float64)
    out = oracle.compose_layers(Ko, So, Vo, planar_to_interleaved(R0), mode=mode, threads=8)
    rows, cols = R0.shape[1:]
    return np.moveaxis(out.reshape(rows, cols, 3), -1, 0)
