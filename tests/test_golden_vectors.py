"""The committed regression vectors (tests/golden/oracle_vectors.json) for the
paths the reference ships no frozen values for: the oracle must keep
producing them (CPU), and the GPU engine must produce them through the C ABI
with no oracle in the loop (GPU)."""
import json
import os
import sys
from pathlib import Path

import pytest

GOLDEN = Path(__file__).parent / 'golden'
sys.path.insert(0, str(GOLDEN))
from cases import CASES  # noqa: E402

VECTORS = json.loads((GOLDEN / 'oracle_vectors.json').read_text())


@pytest.mark.parametrize('name', sorted(CASES))
def test_oracle_reproduces_the_vectors(name):
    import oracle
    new2d = lambda sc: oracle.OracleEngine(sc.n + 512, threads=os.cpu_count() or 1).load_scene(sc)
    new3d = lambda sc, stir=0: oracle.Oracle3D(sc.n, iters=3, threads=os.cpu_count() or 1).load_scene(sc, stir)
    assert CASES[name](new2d, new3d) == VECTORS[name]


@pytest.mark.gpu
@pytest.mark.parametrize('name', sorted(CASES))
def test_gpu_reproduces_the_vectors(name):
    from sunaengine_gb300.engine import Engine
    from sunaengine_gb300.engine3d import Engine3D
    new2d = lambda sc: Engine(max_particles=sc.n + 512, debug=True).load_scene(sc)

    class E3(Engine3D):
        def fnv_hex(self):
            return self.chain()

    new3d = lambda sc, stir=0: E3(max_particles=sc.n, iters=3).load_scene(sc, stir)
    assert CASES[name](new2d, new3d) == VECTORS[name]
