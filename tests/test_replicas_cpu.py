"""Replica fan-out (namsa_gb300/replicas.py) with two gloo ranks on the CPU: the
reference's block split (namsa/msa.py:1015-1022), the ordered gather of uneven
blocks (msa.py:1053-1081), the max-over-ranks step time, the per-rank position
blocks of MSAReplicas, and a rank that leaves between steps (the survivor's
collective fails instead of hanging)."""
import json
import os
import socket
import subprocess
import sys

import pytest

from namsa_gb300 import replicas as R

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _run(scenario, tmp_path, world=2, extra_env=None, timeout=120):
    port = _free_port()
    procs, outs = [], []
    for rank in range(world):
        out = tmp_path / f'{scenario}_{rank}.json'
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                   MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES='')
        env.update(extra_env or {})
        procs.append(subprocess.Popen([sys.executable, os.path.join(HERE, 'replica_worker.py'), scenario, str(out)],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
        outs.append(out)
    logs = []
    for p in procs:
        try:
            logs.append(p.communicate(timeout=timeout)[0].decode(errors='replace'))
        except subprocess.TimeoutExpired:
            p.kill()
            pytest.fail(f'{scenario}: a rank did not finish within {timeout} s')
    return [json.load(open(o)) if o.exists() else None for o in outs], logs


def test_block_parts_follow_the_reference_split():
    assert R.block_parts(1024, 1) == [(0, 1024)]
    assert R.block_parts(1024, 3) == [(0, 341), (341, 682), (682, 1024)]
    assert R.block_parts(5, 2) == [(0, 2), (2, 5)]
    parts = R.block_parts(1000, 8)
    assert parts[0][0] == 0 and parts[-1][1] == 1000
    assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))


@pytest.mark.parametrize('n', [5, 8])
def test_gather_keeps_position_order_with_uneven_blocks(tmp_path, n):
    res, logs = _run('gather', tmp_path, extra_env={'NPOS': str(n)})
    assert res[0] is not None and res[1] is not None, logs
    assert res[0]['full'] == list(range(n))
    assert res[0]['shape'] == [n, 3, 4]
    assert res[1]['full'] is None


def test_max_over_ranks(tmp_path):
    res, logs = _run('max', tmp_path)
    assert [r['max'] for r in res] == [11.0, 11.0], logs


def test_replica_position_blocks(tmp_path):
    res, logs = _run('partition', tmp_path)
    assert res[0] is not None and res[1] is not None, logs
    assert res[0]['block'] == [0.0, 1.0, 2.0] and res[1]['block'] == [3.0, 4.0, 5.0, 6.0]
    assert [r['num_probes'] for r in res] == [3, 4] and res[0]['total'] == 7


def test_dead_peer_fails_the_collective_instead_of_hanging(tmp_path):
    res, logs = _run('dead_peer', tmp_path, timeout=90)
    assert res[0] is not None, logs
    assert res[0]['raised'] is True
