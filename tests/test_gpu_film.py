"""Film output on the GPU (slrgpu_film_to_bmp) against the reference's
ImageSensor::saveImage on the same film: identical BMP headers, and pixel
bytes that agree exactly except where the float exp / pow of the two
libraries differ in the last bit right at an 8-bit step (at most 1 apart, on
at most 0.1 % of the bytes).  The padding bytes of each row are excluded:
the reference leaves them uninitialised."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h", [(37, 23), (64, 16)])
def test_film_bmp_matches_reference(gpu_lib, oracle_lib, tmp_path, w, h):
    rng = np.random.default_rng(w * h)
    film = np.exp(rng.normal(-1.0, 2.0, (h, w, 16))).astype(np.float32)
    film[0, 0] = 0.0                                   # black
    film[1, 1] = 1e6                                   # saturated
    film[2, :, 3] = 0.0                                # a bin empty along a row
    scale, sens = 0.37, 2.5
    ours = str(tmp_path / "gpu.bmp")
    ref = str(tmp_path / "ref.bmp")
    px = gpu_lib.film_to_bmp(film, scale, sens, ours)
    oracle_lib.film_bmp(film, scale, sens, ref)
    a, b = open(ours, "rb").read(), open(ref, "rb").read()
    assert len(a) == len(b) and a[:54] == b[:54]
    row = 3 * w + w % 4
    pa = np.frombuffer(a[54:], np.uint8).reshape(h, row)[:, :3 * w].astype(int)
    pb = np.frombuffer(b[54:], np.uint8).reshape(h, row)[:, :3 * w].astype(int)
    assert np.array_equal(px[:, :3 * w], pa)
    diff = np.abs(pa - pb)
    assert diff.max() <= 1 and (diff > 0).mean() <= 1e-3, (diff.max(), (diff > 0).mean())
    assert pa.min() == 0 and pa.max() == 255
