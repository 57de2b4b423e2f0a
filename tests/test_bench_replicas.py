"""The bench's N > 1 launch path (one process per GPU, replicas, MAX over ranks)
with world_size-2 gloo ranks on the CPU."""
import json
import os
import re
import socket
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def torchrun(args, timeout=300):
    pytest.importorskip('torch')
    env = dict(os.environ, OMP_NUM_THREADS='2')
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node', '2',
           '--master-addr', '127.0.0.1', '--master-port', str(free_port())] + args
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_max_over_ranks_and_barrier(tmp_path):
    script = tmp_path / 'rk.py'
    script.write_text(textwrap.dedent(f'''
        import json, sys
        sys.path.insert(0, {str(ROOT)!r})
        import bench
        ws, rank, local, dist = bench._dist()
        bench._barrier(dist)
        m = bench._max_over_ranks(dist, 10.0 + 5 * rank, local)
        sys.stdout.write(json.dumps({{"rank": rank, "ws": ws, "max": m, "backend": dist.get_backend()}}) + "\\n")
        sys.stdout.flush()
        dist.destroy_process_group()
    '''))
    r = torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    # the two ranks share one stdout, so their lines may arrive run together
    lines = [json.loads(x) for x in re.findall(r'\{[^{}]*\}', r.stdout)]
    assert sorted(l['rank'] for l in lines) == [0, 1]
    assert all(l['ws'] == 2 and l['max'] == 15.0 and l['backend'] == 'gloo' for l in lines)


def test_reference_arm_prints_one_line_from_rank_zero():
    r = torchrun(['bench.py', '--impl', 'reference', '--gpus', '2', '--steps', '1', '--warmup', '3'])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    line = lines[0]
    assert line['impl'] == 'reference' and line['n_gpus'] == 2 and line['value'] > 0
    assert line['e2e']['h2d_bytes_per_step'] == 0 and line['cpu_baseline']['kind'] == 'port'
