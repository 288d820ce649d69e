"""Golden vectors from the reference's own Python implementation,
python/tinypede.py of the Millepede-II sources (local fits by dense
inversion, global matrix and vector, constraints by Lagrange multipliers,
solution and errors by inversion of the bordered matrix).

    python tests/golden/make_golden.py [path to the Millepede-II sources]

For every case the seeded synthetic records are made by the package's
generator (the SHA-256 of the record arrays is stored so a test can see that
it regenerates the same input), written as a C-format Mille file, read back
by tinypede and processed with its Pede class.  Stored per case (.npz):
the label order, the global matrix (packed lower triangle, or for larger
cases its diagonal plus products with seeded probe vectors), the global
vector, the solution and the errors.  tinypede's chi2 scaling factor is set
huge so that it rejects nothing (its rejection test is not pede's).
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
    for k in ("nmod", "minHits", "maxHits"):
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
        p.construct(chi2Factor=1e12)
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


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    sys.path.insert(0, os.path.join(ref, "python"))
    import tinypede
    mp = load_mp()
    for name, c in CASES.items():
        d = case_data(mp, c)
        with tempfile.TemporaryDirectory() as tmp:
            out = run_tinypede(tinypede, mp, d, c, tmp)
        out["record_sha256"] = np.array(record_hash(d))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "npar", len(out["labels"]), "rejects", int(out["nrejects"]),
              "bad", int(out["nbad"]))


if __name__ == "__main__":
    main()
