"""Layout facts of the reference's golden result file CI/refFiles/millepede.res
(written by pede's prtglo with `printcounts`, no errors: formats 110/111,
pede.f90:4548-4600) for tests/test_res_writer.py: the header line, the
shapes of the parameter lines (number of fields, length) with their counts,
and three of the lines (first, middle, last).

    python tests/golden/make_res_layout.py <path to the Millepede-II sources>
    (or the path in the environment variable MILLEPEDE_SOURCES)
"""
import collections
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MILLEPEDE_SOURCES")
    if not src:
        sys.exit("give the Millepede-II sources as argument or in MILLEPEDE_SOURCES")
    with open(os.path.join(src, "CI", "refFiles", "millepede.res")) as f:
        lines = f.read().splitlines()
    body = lines[1:]
    shapes = collections.Counter((len(l.split()), len(l)) for l in body)
    out = {
        "source": "CI/refFiles/millepede.res",
        "header": lines[0],
        "nlines": len(body),
        "shapes": sorted([n, w, c] for (n, w), c in shapes.items()),
        "samples": [body[0], body[len(body) // 2], body[-1]],
    }
    with open(os.path.join(HERE, "millepede_res_layout.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
