"""pairentries (steering `pairentries`, mreqpe > 1; clbits/inbits/ndbits
mpbits.f90:73-142, 182-243, 305-566; the record pairs of loop2
pede.f90:6889-6908 and the measurement-line pairs pede.f90:7036): group
pairs met in fewer than mreqpe records are left out of the sparse matrix and
their updates are dropped, as mupdat drops an element that is not stored
(pede.f90:3172).  pede's own loopbf does not drop them: mgupdt stops when
the first group of a run is not stored (pede.f90:3313-3319), so the drop
rule here is mupdat's.

CPU: the oracle's structure against pair counts taken from the records in
Python; the library's host pass against the oracle (columns and the list of
left-out pairs); measurement-line records always kept; the oracle's data
loop in sparse storage equal to packed storage on every stored element.
GPU: the data loop and a whole job against the oracle."""
import ctypes as C
from collections import Counter

import numpy as np
import pytest

import oracle_ref as orc

i32p, i64p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)


def record_groups(S, recPtr, tinder, glder):
    """sorted variable groups of every record (the measurements' global
    words, as the structure passes read them)"""
    out = []
    for r in range(len(recPtr) - 1):
        end, lg, g = recPtr[r + 1] - 1, recPtr[r], set()
        while lg < end:
            lg += 1
            while tinder[lg] != 0:
                lg += 1
            sl = lg
            lg += 1
            while tinder[lg] != 0:
                lg += 1
            sg = lg
            if sl + 1 == sg and glder[sg] < 0.0:
                lg += int(-glder[sg] + 0.5)
                continue
            while lg < end and tinder[lg + 1] != 0:
                lg += 1
            for w in range(sg + 1, lg + 1):
                v = S.varIndex[tinder[w] - 1]
                if v > 0:
                    g.add(int(S.p2g[v - 1]) if hasattr(S, "p2g") else group_of(S, v))
        out.append(sorted(g))
    return out


def group_of(S, v):
    return int(np.searchsorted(S.aig, v, side="right"))


def pair_counts(groups, inc=None):
    c = Counter()
    for r, g in enumerate(groups):
        for a in range(len(g)):
            for b in range(a + 1):
                c[(g[a], g[b])] += 1 if inc is None else inc[r]
    return c


def stored_pairs(S):
    """group pairs (I, J) of the sparse structure (uncompressed column lists
    or compressed regions, as ijpgrp reads them, pede.f90:5371-5461)"""
    off, col, aig = S.offsets, S.columns, S.aig
    out = set()
    for I in range(1, S.nG + 1):
        kk, ku = off[2 * (I - 1)], off[2 * I] - off[2 * (I - 1)]
        if ku <= 0:
            continue
        if col[kk] != 0:
            for k in range(ku):
                out.add((I, group_of(S, col[kk + k])))
        else:
            for k in range(2, ku - 1, 2):
                o0, g0, o1 = col[kk + k - 2], col[kk + k - 1], col[kk + k]
                J, w = g0, 0
                while w < o1 - o0:
                    out.add((I, J))
                    w += aig[J] - aig[J - 1]
                    J += 1
    return out


def data(mp, name, ntracks, seed):
    return mp.generate(mp.gen_config(name, ntracks=ntracks, seed=seed))


# counters of 2, 3 (fields crossing the oracle's 32-bit words) and 5 bits;
# column lists and compressed regions (telescope), regions only and rows
# left empty when a group's own pair is left out (barrel, broken lines)
CASES = [("telescope", 300, 5, 2), ("telescope", 300, 5, 4), ("telescope", 300, 5, 20),
         ("barrel", 200, 6, 2), ("barrel", 200, 6, 3), ("brokenlines", 300, 7, 2)]


@pytest.mark.parametrize("name,ntracks,seed,mreqpe", CASES)
def test_oracle_structure_keeps_pairs_met_mreqpe_times(mp, name, ntracks, seed, mreqpe):
    d = data(mp, name, ntracks, seed)
    S = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    cnt = pair_counts(record_groups(S, S.recPtr, S.tinder, S.glder))
    kept = {p for p, c in cnt.items() if c >= mreqpe}
    assert 0 < len(kept) < len(cnt)
    assert stored_pairs(S) == kept
    np_ = np.diff(S.aig)
    nmat = S.nVar + sum(np_[I - 1] * np_[J - 1] for I, J in kept)
    assert S.nmatSparse == nmat
    # pairentries 1: every pair met, the structure of the plain pass
    S1 = orc.Structure(d, mreqenf=1, sparse=True)
    assert stored_pairs(S1) == set(cnt)


@pytest.mark.parametrize("name,ntracks,seed,mreqpe", CASES)
def test_host_structure_equals_oracle(mp, name, ntracks, seed, mreqpe):
    d = data(mp, name, ntracks, seed)
    H = mp.HostStructure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    O = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    np.testing.assert_array_equal(H.offsets, O.offsets)
    np.testing.assert_array_equal(H.columns, O.columns)
    assert H.nmatSparse == O.nmatSparse
    cnt = pair_counts(record_groups(O, O.recPtr, O.tinder, O.glder))
    left = sorted(p for p, c in cnt.items() if c < mreqpe)
    np.testing.assert_array_equal(H.suppressed, np.array(left, np.int32).reshape(-1, 2))


def structure_only_record(S, labels):
    """header, measurement value, sigma 1 and the labels as global words
    (total indices), the layout of the structure-only record of a
    measurement line"""
    idx = [int(np.searchsorted(S.labels, l)) + 1 for l in labels]
    return [0, 0, 0] + idx, [0.0, 0.0, 1.0] + [1.0] * len(idx)


def test_measurement_line_pairs_always_kept(mp):
    """records from nrecData on count mreqpe per pair (pede.f90:7036): a
    pair no record holds, and pairs met once, are kept when a measurement
    line links them; host pass = oracle pass"""
    d = data(mp, "telescope", 300, 5)
    mreqpe = 3
    O = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    groups = record_groups(O, O.recPtr, O.tinder, O.glder)
    cnt = pair_counts(groups)
    rare = [p for p, c in cnt.items() if c == 1 and p[0] != p[1]][0]
    lab_of_group = {group_of(O, O.varIndex[t]): O.labels[t] for t in range(O.nTotal) if O.varIndex[t] > 0}
    never = next((I, J) for I in range(2, O.nG + 1) for J in range(1, I) if (I, J) not in cnt)
    lines = [[lab_of_group[rare[0]], lab_of_group[rare[1]]], [lab_of_group[never[0]], lab_of_group[never[1]]]]
    rp, ind, gl = list(O.recPtr), list(O.tinder), list(O.glder)
    for ln in lines:
        w, g = structure_only_record(O, ln)
        ind += w
        gl += g
        rp.append(len(ind))
    rp, ind, gl = np.array(rp, np.int64), np.array(ind, np.int32), np.array(gl)
    nrec, nrecData = len(rp) - 1, len(O.recPtr) - 1
    out = {}
    for side in ("oracle", "host"):
        off = np.zeros(2 * (O.nG + 1), np.int64)
        cap = 1 << 20
        col = np.zeros(cap, np.int32)
        ncolw, nmat, nsup = C.c_int64(), C.c_int64(), C.c_int64()
        if side == "oracle":
            rc = orc.lib().mpref_mpbits(
                C.c_int64(nrec), C.c_int64(nrecData), orc.ptr(rp, i64p), orc.ptr(ind, i32p),
                orc.ptr(gl, f64p), orc.ptr(O.varIndex, i32p), C.c_int32(O.nVar), C.c_int32(O.nG),
                orc.ptr(O.aig, i32p), orc.ptr(O.p2g, i32p), C.c_int32(mreqpe), C.c_int64(cap),
                orc.ptr(off, i64p), orc.ptr(col, i32p), C.byref(ncolw), C.byref(nmat))
            sup = None
        else:
            sup = np.zeros(2 * 100000, np.int32)
            rc = mp.lib().mpgpu_host_mpbits_pairentries(
                C.c_int64(nrec), C.c_int64(nrecData), mp.ptr(rp, i64p), mp.ptr(ind, i32p),
                mp.ptr(gl, f64p), mp.ptr(O.varIndex, i32p), C.c_int32(O.nVar), C.c_int32(O.nG),
                mp.ptr(O.aig, i32p), C.c_int32(mreqpe), C.c_int64(cap), mp.ptr(off, i64p),
                mp.ptr(col, i32p), C.byref(ncolw), C.byref(nmat), C.c_int64(100000), mp.ptr(sup, i32p),
                C.byref(nsup))
            sup = sup[:2 * nsup.value].reshape(-1, 2)
        assert rc == 0
        out[side] = (off, col[:ncolw.value].copy(), nmat.value, sup)
    np.testing.assert_array_equal(out["host"][0], out["oracle"][0])
    np.testing.assert_array_equal(out["host"][1], out["oracle"][1])
    assert out["host"][2] == out["oracle"][2]

    class V:
        pass
    v = V()
    v.offsets, v.columns, v.aig, v.nG = out["oracle"][0], out["oracle"][1], O.aig, O.nG
    st = stored_pairs(v)
    for I, J in (rare, never):
        assert (max(I, J), min(I, J)) in st
    kept = {p for p, c in cnt.items() if c >= mreqpe}
    assert kept < st
    left = {tuple(p) for p in out["host"][3]}
    assert (max(rare), min(rare)) not in left and left.isdisjoint(st)


def test_host_structure_capacity_retry(mp):
    """-1 with the sizes when the arrays are short, as the other passes"""
    d = data(mp, "barrel", 200, 6)
    O = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=2)
    nrec = len(O.recPtr) - 1
    off = np.zeros(2 * (O.nG + 1), np.int64)
    col = np.zeros(4, np.int32)
    sup = np.zeros(2, np.int32)
    ncolw, nmat, nsup = C.c_int64(), C.c_int64(), C.c_int64()
    rc = mp.lib().mpgpu_host_mpbits_pairentries(
        C.c_int64(nrec), C.c_int64(nrec), mp.ptr(O.recPtr, i64p), mp.ptr(O.tinder, i32p),
        mp.ptr(O.glder, f64p), mp.ptr(O.varIndex, i32p), C.c_int32(O.nVar), C.c_int32(O.nG),
        mp.ptr(O.aig, i32p), C.c_int32(2), C.c_int64(len(col)), mp.ptr(off, i64p), mp.ptr(col, i32p),
        C.byref(ncolw), C.byref(nmat), C.c_int64(1), mp.ptr(sup, i32p), C.byref(nsup))
    assert rc == -1
    assert ncolw.value == len(O.columns) and nmat.value == O.nmatSparse
    cnt = pair_counts(record_groups(O, O.recPtr, O.tinder, O.glder))
    assert nsup.value == sum(1 for c in cnt.values() if c < 2)
    np.testing.assert_array_equal(off, O.offsets)


def sparse_elements(S):
    """(row, column, position in globalMatD) of every stored off-diagonal
    element, 1-based parameter indices (ijadd, pede.f90:5498-5537)"""
    off, col, aig = S.offsets, S.columns, S.aig
    rows, cols, pos = [], [], []
    for I in range(1, S.nG + 1):
        kk, ll = off[2 * (I - 1)], off[2 * (I - 1) + 1]
        ku = off[2 * I] - kk
        if ku <= 0:
            continue
        np_ = aig[I] - aig[I - 1]
        if col[kk] != 0:
            for a in range(np_):
                for k in range(ku):
                    rows.append(aig[I - 1] + a)
                    cols.append(col[kk + k])
                    pos.append(ll + a * ku + k)
        else:
            for k in range(2, ku - 1, 2):
                o0, g0, o1 = col[kk + k - 2], col[kk + k - 1], col[kk + k]
                for a in range(np_):
                    for w in range(o1 - o0):
                        rows.append(aig[I - 1] + a)
                        cols.append(aig[g0 - 1] + w)
                        pos.append(ll + o0 * np_ + a * (o1 - o0) + w)
    r, c, p = np.array(rows), np.array(cols), np.array(pos)
    keep = c < r   # lower triangle without the diagonal (kept apart)
    return r[keep], c[keep], p[keep]


@pytest.mark.parametrize("name,ntracks,seed,mreqpe", [("telescope", 300, 5, 3), ("barrel", 60, 6, 2)])
def test_oracle_loop_drops_only_left_out_pairs(mp, name, ntracks, seed, mreqpe):
    """the oracle's data loop in sparse storage with the drop rule equals
    the packed loop on every stored element and on the diagonal and vector
    (the same sums in the same record order); without the rule a left-out
    pair is error 23"""
    d = data(mp, name, ntracks, seed)
    S = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    gpar = np.zeros(S.nTotal)
    sp = S.loopbf(gpar, matsto=2)
    pk = S.loopbf(gpar, matsto=1)
    assert sp["rc"] == 0 and pk["rc"] == 0
    np.testing.assert_array_equal(sp["status"], pk["status"])
    np.testing.assert_array_equal(sp["gvec"], pk["gvec"])
    n = S.nVar
    i = np.arange(1, n + 1)
    np.testing.assert_array_equal(sp["matD"][:n], pk["matD"][(i * i - i) // 2 + i - 1])
    r, c, p = sparse_elements(S)
    np.testing.assert_array_equal(sp["matD"][p], pk["matD"][(r * r - r) // 2 + c - 1])
    # the packed matrix holds elements that the sparse one left out
    dropped = np.ones(len(pk["matD"]), bool)
    dropped[(i * i - i) // 2 + i - 1] = False
    dropped[(r * r - r) // 2 + c - 1] = False
    assert np.count_nonzero(pk["matD"][dropped]) > 0
    assert S.loopbf(gpar, matsto=2, mreqpe=1)["rc"] == 23


def test_oracle_job_pairentries(mp):
    """whole oracle job: pairentries changes the sparse solution (pairs are
    dropped) and leaves full storage alone (pede reads it for sparse
    storage only, pede.f90:6564)"""
    d = data(mp, "telescope", 400, 11)
    res = {}
    for matsto, mreqpe in ((2, 1), (2, 3), (1, 1), (1, 3)):
        st = orc.make_steer(metsol=4, matsto=matsto, mitera=1, mrestl=1e-14, itnlim=4000, mreqpe=mreqpe)
        o = orc.run(d, st)
        assert o["rc"] == 0
        res[(matsto, mreqpe)] = o["parameter"]
    scale = np.max(np.abs(res[(2, 1)]))
    assert np.max(np.abs(res[(2, 3)] - res[(2, 1)])) > 1e-6 * scale
    np.testing.assert_array_equal(res[(1, 3)], res[(1, 1)])


def close(a, b, tol=1e-12):
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale if a.size else 0.0
    assert err <= tol, f"max rel diff {err:.3e} > {tol:.1e}"


@pytest.mark.gpu
@pytest.mark.parametrize("name,ntracks,seed,mreqpe", [("barrel", 3000, 6, 2), ("telescope", 600, 5, 3)])
def test_gpu_loop_drops_left_out_pairs(mp, name, ntracks, seed, mreqpe):
    """device data loop with the left-out pairs' blocks in the accumulation
    table (mpgpu_set_suppressed_pairs) against the oracle's loop with the
    drop rule: decisions exact, matrix and vector 1e-12 relative"""
    d = data(mp, name, ntracks, seed)
    H = mp.HostStructure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    O = orc.Structure(d, mreqenf=1, sparse=True, mreqpe=mreqpe)
    assert len(H.suppressed) > 0
    gpar = np.zeros(H.nTotal)
    o = O.loopbf(gpar, matsto=2)
    with mp.Context() as ctx:
        ctx.set_layout(H, 2)
        ctx.upload(H)
        g = ctx.loopbf(gpar)
        g["matD"] = ctx.matrix()
        g["status"] = ctx.status()
    assert o["rc"] == 0
    np.testing.assert_array_equal(g["status"], o["status"])
    np.testing.assert_array_equal(g["gcnt"], o["gcnt"])
    close(g["gvec"], o["gvec"])
    close(g["matD"], o["matD"])


@pytest.mark.gpu
def test_gpu_job_pairentries(mp):
    """whole job (MINRES, sparse, pairentries 3) through mpgpu_pede_run
    against the oracle's job driver"""
    import test_gpu_pede as T
    d = data(mp, "telescope", 400, 11)
    st = orc.make_steer(metsol=4, matsto=2, mitera=2, mrestl=1e-14, itnlim=4000, mreqpe=3)
    g = T.gpu_job(mp, orc, d, st)
    o = orc.run(d, st)
    assert g["rc"] == 0 and o["rc"] == 0
    np.testing.assert_array_equal(g["labels"], o["labels"])
    np.testing.assert_array_equal(g["counts"], o["counts"])
    assert g["nrej"] == o["nrej"]
    scale = np.max(np.abs(o["parameter"]))
    assert np.max(np.abs(g["parameter"] - o["parameter"])) <= 1e-9 * scale


def test_host_structure_bad_arguments(mp):
    """status 44 for arguments the pass cannot use (no groups, no
    parameters, a list capacity without a list)"""
    rp = np.array([0, 1], np.int64)
    ind = np.zeros(1, np.int32)
    gl = np.zeros(1)
    vi = np.ones(1, np.int32)
    aig = np.array([1, 2], np.int32)
    off = np.zeros(4, np.int64)
    col = np.zeros(4, np.int32)
    ncolw, nmat, nsup = C.c_int64(), C.c_int64(), C.c_int64()
    L = mp.lib()

    def call(nVar, nG, capSup, sup):
        return L.mpgpu_host_mpbits_pairentries(
            C.c_int64(1), C.c_int64(1), mp.ptr(rp, i64p), mp.ptr(ind, i32p), mp.ptr(gl, f64p),
            mp.ptr(vi, i32p), C.c_int32(nVar), C.c_int32(nG), mp.ptr(aig, i32p), C.c_int32(2),
            C.c_int64(4), mp.ptr(off, i64p), mp.ptr(col, i32p), C.byref(ncolw), C.byref(nmat),
            C.c_int64(capSup), sup, C.byref(nsup))
    assert call(1, 0, 0, None) == 44
    assert call(0, 1, 0, None) == 44
    assert call(1, 1, 8, None) == 44
    assert call(1, 1, 0, None) == 0 and nsup.value == 0 and nmat.value == 1
