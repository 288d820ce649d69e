"""Mille binary files through mpgpu_read_mille (no device): C and Fortran
framing, double and float words, gzip-compressed files, several files with
the file index per record, a record limit per file, and a damaged file
(status 20)."""
import gzip
import shutil

import numpy as np
import pytest


def write(path, recPtr, inder, glder, fortran, double):
    with open(path, "wb") as f:
        for r in range(len(recPtr) - 1):
            a, b = recPtr[r], recPtr[r + 1]
            n = b - a
            g = glder[a:b].astype(np.float64 if double else np.float32)
            payload = np.array([-2 * n if double else 2 * n], np.int32).tobytes() + g.tobytes() + \
                inder[a:b].astype(np.int32).tobytes()
            if fortran:
                f.write(np.array([len(payload)], np.int32).tobytes() + payload +
                        np.array([len(payload)], np.int32).tobytes())
            else:
                f.write(payload)


@pytest.mark.parametrize("fortran", [False, True])
@pytest.mark.parametrize("double", [False, True])
def test_read_formats(mp, tmp_path, fortran, double):
    d = mp.generate(mp.gen_config("telescope", ntracks=300, seed=9))
    p = str(tmp_path / "a.bin")
    write(p, d["recPtr"], d["inder"], d["glder"], fortran, double)
    recPtr, inder, glder, recFile = mp.read_mille([p])
    np.testing.assert_array_equal(recPtr, d["recPtr"])
    np.testing.assert_array_equal(inder, d["inder"])
    want = d["glder"] if double else d["glder"].astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(glder, want)
    assert np.all(recFile == 1)


def test_several_files_and_limit(mp, tmp_path):
    d1 = mp.generate(mp.gen_config("telescope", ntracks=50, seed=1))
    d2 = mp.generate(mp.gen_config("barrel", ntracks=40, seed=2))
    p1, p2 = str(tmp_path / "c.bin"), str(tmp_path / "f.bin")
    write(p1, d1["recPtr"], d1["inder"], d1["glder"], False, True)
    write(p2, d2["recPtr"], d2["inder"], d2["glder"], True, True)
    recPtr, inder, glder, recFile = mp.read_mille([p1, p2], max_rec=30)
    assert len(recPtr) - 1 == 60
    np.testing.assert_array_equal(recFile, [1] * 30 + [2] * 30)
    n1 = d1["recPtr"][30]
    np.testing.assert_array_equal(inder[:n1], d1["inder"][:n1])
    np.testing.assert_array_equal(glder[n1:recPtr[-1]], d2["glder"][:d2["recPtr"][30]])


def test_damaged_file(mp, tmp_path):
    d = mp.generate(mp.gen_config("telescope", ntracks=20, seed=3))
    p = str(tmp_path / "t.bin")
    write(p, d["recPtr"], d["inder"], d["glder"], False, True)
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-10])
    with pytest.raises(RuntimeError, match="20"):
        mp.read_mille([p])


@pytest.mark.parametrize("fortran", [False, True])
def test_read_gzip(mp, tmp_path, fortran):
    """A gzip-compressed file (recognised by its first bytes) reads like the
    plain one, also mixed with a plain file."""
    d = mp.generate(mp.gen_config("barrel", ntracks=200, seed=4))
    plain = str(tmp_path / "p.bin")
    write(plain, d["recPtr"], d["inder"], d["glder"], fortran, True)
    packed = str(tmp_path / "p.bin.gz")
    with open(plain, "rb") as src, gzip.open(packed, "wb") as dst:
        shutil.copyfileobj(src, dst)
    a = mp.read_mille([plain])
    b = mp.read_mille([packed])
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    recPtr, inder, glder, recFile = mp.read_mille([packed, plain], max_rec=50)
    assert len(recPtr) - 1 == 100
    np.testing.assert_array_equal(recFile, [1] * 50 + [2] * 50)
    n = d["recPtr"][50]
    np.testing.assert_array_equal(inder[:n], d["inder"][:n])
    np.testing.assert_array_equal(inder[n:], d["inder"][:n])


def test_damaged_gzip(mp, tmp_path):
    d = mp.generate(mp.gen_config("telescope", ntracks=20, seed=3))
    plain = str(tmp_path / "t.bin")
    write(plain, d["recPtr"], d["inder"], d["glder"], False, True)
    raw = gzip.compress(open(plain, "rb").read()[:-10])
    p = str(tmp_path / "t.bin.gz")
    open(p, "wb").write(raw)
    with pytest.raises(RuntimeError, match="20"):
        mp.read_mille([p])
