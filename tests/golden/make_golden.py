"""Golden vectors from the reference's own Python implementation,
python/tinypede.py of the Millepede-II sources (local fits by dense
inversion, global matrix and vector, constraints by Lagrange multipliers,
solution and errors by inversion of the bordered matrix).

    python tests/golden/make_golden.py <path to the Millepede-II sources>
    (or the path in the environment variable MILLEPEDE_SOURCES)

For every case the seeded synthetic records are made by the package's
generator (the SHA-256 of the record arrays is stored so a test can see that
it regenerates the same input), written as a C-format Mille file, read back
by tinypede and processed with its Pede class.  Stored per case (.npz):
the label order, the global matrix (packed lower triangle, or for larger
cases its diagonal plus products with seeded probe vectors), the global
vector, the solution and the errors.

Rejections: tinypede rejects a local fit when prob(chi2 / f, ndf) < 0.0027,
pede when chi2 > chicut * chindl(3, ndf) * ndf (pede.f90:4106-4131), whose
table reproduces the same 3-sigma quantile to 4e-5.  With f = chicut the
two reject the same records unless a chi2 lies within that tolerance of the
cut, so a case with rejections checks (with tinypede's own record reader)
that every record's chi2 is at least 1e-3 away from its cut.  The other
cases set f huge so that nothing is rejected.
"""
import contextlib
import hashlib
import importlib.util
import io
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# name: generator config, tinypede entries cut, fixed labels, constraints,
#       matrix stored in full (else diagonal + probe products)
CASES = {
    "telescope_con": dict(kind="telescope", ntracks=2000, seed=11, entries=25, fixed=(),
                          constraints=True, full=True),
    "telescope_fix": dict(kind="telescope", ntracks=2000, seed=12, entries=25,
                          fixed=tuple(range(1, 21)) + tuple(range(181, 201)),
                          constraints=False, full=True),
    "brokenlines_band": dict(kind="brokenlines", ntracks=60, seed=13, entries=1, fixed=(),
                             constraints=False, full=False, nmod=288, minHits=6, maxHits=12),
    # records with outlier hits, rejected by the chi2 cut of the first loop
    "telescope_rej": dict(kind="telescope", ntracks=3000, seed=14, entries=25, fixed=(),
                          constraints=False, full=True, outlierFrac=0.02, chicut=30.0),
    # the barrel (6 dof per module): mpbits-sparse storage on the device
    "barrel_sparse": dict(kind="barrel", ntracks=3000, seed=15, entries=1, fixed=(),
                          constraints=False, full=False, nmod=300, sparse=True),
}
NPROBE = 4


def load_mp():
    spec = importlib.util.spec_from_file_location(
        "mpgpu_golden", os.path.join(ROOT, "millepede-ii_gb300", "mpgpu.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def case_data(mp, c):
    cfg = mp.gen_config(c["kind"], ntracks=c["ntracks"], seed=c["seed"])
    for k in ("nmod", "minHits", "maxHits", "outlierFrac"):
        if k in c:
            setattr(cfg, k, c[k])
    return mp.generate(cfg)


def record_hash(d):
    h = hashlib.sha256()
    for k in ("recPtr", "inder", "glder"):
        h.update(np.ascontiguousarray(d[k]).tobytes())
    return h.hexdigest()


def probes(n):
    return np.random.default_rng(2024).normal(size=(NPROBE, n))


def run_tinypede(tinypede, mp, d, c, tmp):
    binf = os.path.join(tmp, "data.bin")
    conf = os.path.join(tmp, "con.txt")
    mp.write_mille_c(binf, d["recPtr"], d["inder"], d["glder"])
    with open(conf, "w") as f:
        if c["constraints"]:
            cs, cl, cc = d["conStart"], d["conLabel"], d["conCoef"]
            for k in range(d["ncon"]):
                f.write("Constraint 0.0\n")
                for q in range(cs[k], cs[k + 1]):
                    f.write(f"{int(cl[q])} {float(cc[q])!r}\n")
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        p = tinypede.Pede()
        p.addBinaryFile(binf, len(d["recPtr"]) - 1, "C")
        p.defineParameters(c["entries"], list(c["fixed"]))
        p.addConstraints(conf)
        p.construct(chi2Factor=c.get("chicut", 1e12))
    npar = p._Pede__numPar
    M = p._Pede__matrix
    vec = p._Pede__vector[:npar].copy()
    A = M[:npar, :npar].copy()
    cov = np.linalg.inv(M)
    sol = cov @ p._Pede__vector
    idx = p._Pede__parIndices
    labels = np.array(sorted(idx, key=lambda l: idx[l]), np.int32)
    diag = np.diag(cov)[:npar]
    err = np.where(diag > 0, np.sqrt(np.abs(diag)), -np.sqrt(np.abs(diag)))
    out = dict(labels=labels, vector=vec, solution=sol[:npar], error=err,
               nrejects=np.int64(p._Pede__numRejects), nbad=np.int64(p._Pede__numBad),
               diag=np.diag(A).copy(), probe=A @ probes(npar).T)
    if c["full"]:
        out["packed"] = A[np.tril_indices(npar)]
    return out


def cut_margin(tinypede, mp, d, c, tmp):
    """Smallest relative distance of a record's local-fit chi2 from the cut
    f * q3(ndf) (q3: the 3-sigma quantile), over the records, read with
    tinypede's record reader and fitted by plain least squares."""
    from scipy.stats import chi2
    binf = os.path.join(tmp, "margin.bin")
    mp.write_mille_c(binf, d["recPtr"], d["inder"], d["glder"])
    f = c["chicut"]
    best = np.inf
    with open(binf, "rb") as fh:
        for _ in range(len(d["recPtr"]) - 1):
            rec = tinypede.MilleRecord()
            rec.readRecord(fh, "C")
            rows, meas, wts = [], [], []
            nloc = 0
            while rec.moreData():
                if rec.specialDataTag() >= 0:
                    continue
                aMeas, aPrec, indLocal, derLocal, _, _ = rec.getData()
                rows.append(dict(zip(indLocal, derLocal)))
                meas.append(aMeas)
                wts.append(aPrec)
                nloc = max(nloc, max(indLocal))
            L = np.zeros((len(rows), nloc))
            for i, r in enumerate(rows):
                for k, v in r.items():
                    L[i, k - 1] = v
            w = np.array(wts)
            m = np.array(meas)
            q = np.linalg.solve(L.T @ (w[:, None] * L), L.T @ (w * m))
            res = m - L @ q
            c2 = float(res @ (w * res))
            ndf = len(rows) - nloc
            cut = f * chi2.ppf(1.0 - 0.0027, ndf)
            best = min(best, abs(c2 - cut) / cut)
    return best


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MILLEPEDE_SOURCES")
    if not ref:
        sys.exit("usage: make_golden.py <path to the Millepede-II sources> (or set MILLEPEDE_SOURCES)")
    sys.path.insert(0, os.path.join(ref, "python"))
    import tinypede
    mp = load_mp()
    for name, c in CASES.items():
        d = case_data(mp, c)
        with tempfile.TemporaryDirectory() as tmp:
            if "chicut" in c:
                margin = cut_margin(tinypede, mp, d, c, tmp)
                assert margin > 1e-3, f"{name}: a chi2 lies {margin:.1e} from its cut"
                print(name, "smallest relative distance of a chi2 from its cut", f"{margin:.2e}")
            out = run_tinypede(tinypede, mp, d, c, tmp)
        out["record_sha256"] = np.array(record_hash(d))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "npar", len(out["labels"]), "rejects", int(out["nrejects"]),
              "bad", int(out["nbad"]))


if __name__ == "__main__":
    main()
