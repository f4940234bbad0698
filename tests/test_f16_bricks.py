"""The FP16 brick grid format (SDFC_STORAGE_F16_BRICKS), host-only codec of libsdfcontact:
no GPU needed.  The codes are pinned bit for bit to a NumPy restatement of the encoder (FP16
rounding to nearest even, as numpy.float16), and the decoded grid stays within FP16's relative
precision of each node's distance from its brick's offset."""
import numpy as np

from conftest import submodule


def numpy_encode(v):
    nk, nj, ni = v.shape
    nbx, nby, nbz = (ni + 7) // 8, (nj + 7) // 8, (nk + 7) // 8
    codes = np.zeros(nbx * nby * nbz * 512, dtype=np.uint16)
    so = np.zeros((nbx * nby * nbz, 2), dtype=np.float32)
    for bz in range(nbz):
        for by in range(nby):
            for bx in range(nbx):
                b = bx + nbx * (by + nby * bz)
                kk = np.minimum(8 * bz + np.arange(8), nk - 1)
                jj = np.minimum(8 * by + np.arange(8), nj - 1)
                ii = np.minimum(8 * bx + np.arange(8), ni - 1)
                blk = v[np.ix_(kk, jj, ii)]  # [k][j][i]
                lo, hi = blk.min(), blk.max()
                off = np.float32(0.0) if lo <= 0.0 <= hi else np.float32(lo if lo > 0 else hi)
                amax = max(abs(hi - float(off)), abs(lo - float(off)))
                scale = np.float32(amax / 32768.0) if amax > 0 else np.float32(1.0)
                so[b] = (scale, off)
                q = ((blk - float(off)) / float(scale)).astype(np.float32).astype(np.float16)
                codes[b * 512:(b + 1) * 512] = q.view(np.uint16).ravel()  # i + 8 j + 64 k
    return codes, so


def test_codec_matches_numpy_and_bounds_error():
    W = submodule("workloads")
    S = submodule("sdfc")
    g = W.sample_grid(W.socket_sdf, [-1, -1, -1], [1, 1, 1], 37, pad=0.1)  # 37^3: partial bricks
    v = g.values[:, :29, :]  # uneven extents (nk, nj, ni) = (37, 29, 37)
    v = np.ascontiguousarray(v)
    codes, so = S.f16_brick_encode(v)
    rc, rso = numpy_encode(v)
    assert np.array_equal(codes, rc)
    assert np.array_equal(so, rso)
    dec = S.f16_brick_decode(codes, so, v.shape)
    nk, nj, ni = v.shape
    nbx, nby = (ni + 7) // 8, (nj + 7) // 8
    K, J, I = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    b = (I >> 3) + nbx * ((J >> 3) + nby * (K >> 3))
    off = so[b, 1].astype(np.float64)
    scale = so[b, 0].astype(np.float64)
    # FP16 keeps 11 significant bits; the FP32 quotient adds one FP32 rounding, the FP32 decode
    # (fmaf(scale, code, offset)) another, of the decoded value
    bound = np.abs(v - off) * 2.0 ** -11 * 1.001 + scale * 2.0 ** -24 + np.abs(dec) * 2.0 ** -24 + 1e-300
    assert np.all(np.abs(dec - v) <= bound)
    # bricks the surface crosses keep offset 0, so values near 0 keep relative precision
    crossing = (v.min() < 0 < v.max())
    assert crossing and np.any(so[:, 1] == 0.0)
    near = np.abs(v) < 0.02
    assert np.all(np.abs(dec[near] - v[near]) <= np.abs(v[near]) * 2.0 ** -11 * 1.001 + scale[near] * 2.0 ** -24
                  + np.abs(dec[near]) * 2.0 ** -24)
