"""Pixel table of a band (the cooler writer's pixel order), oracle side.

The oracle restates Cooler::write_or_append_cmatrix_to_file's pixel loop
(src/libmodle_io/cooler_write_impl.hpp:275-316); here it is checked against an independent
numpy formulation (non-zero entries of the dense upper band, sorted by (bin1, bin2)) on bands
of many shapes, including the edge cases the writer handles: rows past the last column,
an all-zero band, a band narrower than one row and an empty band.
"""

import numpy as np
import pytest

from _harness import oracle_pixels, random_band


def numpy_pixels(band, nrows, ncols, bin_offset):
    b = band.reshape(ncols, nrows)  # b[j, r]: column j (bin2), row r = j - i
    j, r = np.nonzero(b)
    i = j - r
    order = np.lexsort((j, i))
    i, j = i[order], j[order]
    cnt = b[j, j - i]
    offs = np.searchsorted(i, np.arange(ncols + 1), side="left").astype(np.uint64)
    return offs, (i + bin_offset).astype(np.int64), (j + bin_offset).astype(np.int64), cnt


@pytest.mark.parametrize("nrows,ncols,density", [(600, 2000, 0.3), (7, 5, 0.9), (1, 50, 0.5),
                                                 (50, 1, 1.0), (16, 16, 0.0), (3, 0, 0.5),
                                                 (40, 300, 1.0)])
def test_oracle_pixels_match_numpy(nrows, ncols, density):
    rng = np.random.default_rng(nrows * 1000 + ncols)
    band = random_band(rng, nrows, ncols, density)
    got = oracle_pixels(band, nrows, ncols, bin_offset=12345)
    want = numpy_pixels(band, nrows, ncols, 12345)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    assert int(got[0][-1]) == int(np.count_nonzero(band))
