"""Host-side structure (label table, entries, parameter groups, mpbits
sparse layout) against the oracle's literal restatement: bit-exact."""
import numpy as np
import pytest


def _small(mp, name, ntracks, seed=7):
    return mp.generate(mp.gen_config(name, ntracks=ntracks, seed=seed))


@pytest.mark.parametrize("name,ntracks", [("telescope", 3000), ("barrel", 4000)])
def test_structure_matches_oracle(mp, orc, name, ntracks):
    d = _small(mp, name, ntracks)
    H = mp.HostStructure(d, mreqenf=5)
    O = orc.Structure(d, mreqenf=5)
    assert H.nTotal == O.nTotal and H.nVar == O.nVar and H.nG == O.nG
    np.testing.assert_array_equal(H.labels, O.labels)
    np.testing.assert_array_equal(H.counter, O.counter)
    np.testing.assert_array_equal(H.varIndex, O.varIndex)
    np.testing.assert_array_equal(H.totGroup, O.totGroup)
    np.testing.assert_array_equal(H.aig, O.aig)
    np.testing.assert_array_equal(H.tinder, O.tinder)
    np.testing.assert_array_equal(H.offsets, O.offsets)
    np.testing.assert_array_equal(H.columns[:H.ncolw], O.columns[:O.ncolw])
    assert H.nmatSparse == O.nmatSparse


def test_groups_random_equations(mp, orc):
    """Random equation structures: parameter groups and entries agree with the
    literal pargrp restatement."""
    rng = np.random.default_rng(11)
    for trial in range(20):
        nlab = int(rng.integers(5, 40))
        recs_i, recs_d, ptrs = [], [], [0]
        for r in range(int(rng.integers(3, 30))):
            ii, dd = [0], [0.0]
            for m in range(int(rng.integers(1, 5))):
                ii += [0, 1]
                dd += [rng.normal(), 1.0]
                k = int(rng.integers(1, 6))
                labs = sorted(set(int(x) for x in rng.integers(1, nlab + 1, k)))
                ii += [0]
                dd += [0.1]
                for lab in labs:
                    ii.append(lab * 3)
                    dd.append(0.0 if rng.random() < 0.1 else float(rng.normal()))
            recs_i += ii
            recs_d += dd
            ptrs.append(len(recs_i))
        d = dict(recPtr=np.array(ptrs, np.int64), inder=np.array(recs_i, np.int32),
                 glder=np.array(recs_d, np.float64))
        H = mp.HostStructure(d, mreqenf=1, sparse=True)
        O = orc.Structure(d, mreqenf=1, sparse=True)
        np.testing.assert_array_equal(H.labels, O.labels)
        np.testing.assert_array_equal(H.counter, O.counter)
        np.testing.assert_array_equal(H.totGroup, O.totGroup)
        np.testing.assert_array_equal(H.varIndex, O.varIndex)
        np.testing.assert_array_equal(H.offsets, O.offsets)
        np.testing.assert_array_equal(H.columns[:H.ncolw], O.columns[:O.ncolw])


def test_labels_status_codes(mp):
    """mpgpu_host_labels: -20 for a measurement without its second marker,
    -23 for a label <= 0 among the global words, -1 beyond the capacity."""
    d = mp.generate(mp.gen_config("telescope", ntracks=50, seed=8))
    zeros = [q for q in range(int(d["recPtr"][3]) + 1, int(d["recPtr"][4])) if d["inder"][q] == 0]
    bad = dict(d, inder=d["inder"].copy())
    bad["inder"][zeros[-1]] = 3
    neg = dict(d, inder=d["inder"].copy())
    neg["inder"][zeros[-1] + 1] = -4
    for data, code in ((bad, "-20"), (neg, "-23")):
        with pytest.raises(RuntimeError, match=f"failed \\({code}\\)"):
            mp.HostStructure(data, mreqenf=1, sparse=False)
    import ctypes as C
    L = mp.lib()
    i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
    a = [np.zeros(4, np.int32) for _ in range(3)]
    cnt = np.zeros(4, np.int64)
    nv, ng = C.c_int32(), C.c_int32()
    rc = L.mpgpu_host_labels(C.c_int64(len(d["recPtr"]) - 1), d["recPtr"].ctypes.data_as(i64p),
                             d["inder"].ctypes.data_as(i32p), d["glder"].ctypes.data_as(f64p),
                             C.c_int32(0), None, C.c_int32(0), None, None, C.c_int32(1), C.c_int32(4),
                             a[0].ctypes.data_as(i32p), cnt.ctypes.data_as(i64p), a[1].ctypes.data_as(i32p),
                             a[2].ctypes.data_as(i32p), C.byref(nv), C.byref(ng))
    assert rc == -1
