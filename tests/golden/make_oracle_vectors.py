"""Record the oracle's answers for the build-defined regression cases
(cases.py) in oracle_vectors.json. Run by hand after a deliberate change to
the oracle; the tests replay these values on the oracle and on the GPU.

    python tests/golden/make_oracle_vectors.py
"""
import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parents[1]))

import oracle  # noqa: E402
from cases import CASES  # noqa: E402


def new2d(sc):
    return oracle.OracleEngine(sc.n + 512, threads=os.cpu_count() or 1).load_scene(sc)


def new3d(sc, stir=0):
    return oracle.Oracle3D(sc.n, iters=3, threads=os.cpu_count() or 1).load_scene(sc, stir)


if __name__ == '__main__':
    out = {name: f(new2d, new3d) for name, f in CASES.items()}
    (HERE / 'oracle_vectors.json').write_text(json.dumps(out, indent=2, sort_keys=True) + '\n')
    print(json.dumps(out, indent=2))
