"""The device Zernike table (Noll index -> (n, m), radial coefficients) against the oracle.

dlx_zernike_table is host code of the library, so this runs without a GPU.
"""

import numpy as np

from oracle import dlux_oracle as O


def test_noll_map_and_radial_coefficients():
    from dlux_gb300 import _lib
    lib = _lib.load()
    for start in (1, 61):
        js = np.arange(start, start + 60, dtype=np.int32)
        K = len(js)
        n = np.zeros(K, np.int32)
        m = np.zeros(K, np.int32)
        c = np.zeros((K, 9), np.float32)
        _lib.check(lib.dlx_zernike_table(js.ctypes.data, K, n.ctypes.data, m.ctypes.data,
                                         c.ctypes.data))
        for i, j in enumerate(js):
            nn, mm = O.noll_indices(int(j))
            assert (nn, mm) == (n[i], m[i]), j
            cc, _ = O.zernike_factors(int(j))
            nk = (nn - abs(mm)) // 2 + 1
            np.testing.assert_allclose(c[i, :nk], cc[:nk], rtol=1e-7)
            assert not c[i, nk:].any()


def test_table_rejects_bad_indices():
    import pytest
    from dlux_gb300 import _lib
    lib = _lib.load()
    bad = np.array([0], np.int32)
    with pytest.raises(ValueError, match="greater than 0"):
        _lib.check(lib.dlx_zernike_table(bad.ctypes.data, 1, None, None, None))
    too_many = np.arange(1, 70, dtype=np.int32)
    with pytest.raises(ValueError, match="terms"):
        _lib.check(lib.dlx_zernike_table(too_many.ctypes.data, 69, None, None, None))


def test_oracle_soft_circle_and_transform():
    coords = O.pixel_coords(64, 1.0)
    t = O.soft_circle(coords, 0.3, 0.02)
    assert t.min() == 0.0 and t.max() == 1.0
    moved = O.coord_transform(coords, translation=(0.1, 0.0))
    tm = O.soft_circle(moved, 0.3, 0.02)
    # the disk moved to +x: its centre of light shifts by the translation
    xs = coords[0]
    assert abs((tm * xs).sum() / tm.sum() - 0.1) < 2e-3
