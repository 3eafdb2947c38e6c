"""One rank of the CPU (gloo) replica tests in tests/test_replicas_cpu.py.

Usage: python tests/replica_worker.py <scenario> <out.json>, with RANK,
WORLD_SIZE, MASTER_ADDR and MASTER_PORT in the environment.  Writes what the
rank observed to out.json.
"""
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from namsa_gb300 import replicas as R  # noqa: E402


def main():
    scenario, out = sys.argv[1], sys.argv[2]
    rank, world = R.init_from_env(backend='gloo', timeout_s=20)
    res = {'rank': rank, 'world': world}
    if scenario == 'gather':
        n = int(os.environ.get('NPOS', '5'))
        parts = R.block_parts(n, world)
        a, b = parts[rank]
        # each position's "CBED" carries its global index
        local = np.arange(a, b, dtype=np.float32)[:, None, None] * np.ones((1, 3, 4), np.float32)
        full = R.gather_blocks(local, parts)
        res['full'] = None if full is None else full[:, 0, 0].tolist()
        res['shape'] = None if full is None else list(full.shape)
    elif scenario == 'max':
        res['max'] = R.max_over_ranks(10.0 + rank)
    elif scenario == 'partition':
        from oracle import msa_oracle as O
        sim = R.MSAReplicas(200, 30e-3, O.si_supercell(2, 2, 2), sampling=np.array([64, 64]), debye_waller=False)
        pos = np.stack([np.arange(7), -np.arange(7)], 1).astype(np.float32)
        sim.set_probe_positions(pos)
        res['block'] = sim.probe_positions[:, 0].tolist()
        res['num_probes'] = int(sim.num_probes)
        res['total'] = int(sim.total_num_probes)
    elif scenario == 'dead_peer':
        if rank == 1:
            os._exit(0)  # leaves between steps, with nothing in flight
        try:
            R.gather_blocks(np.zeros((1, 2, 2), np.float32), R.block_parts(2, world))
            res['raised'] = False
        except Exception as e:  # noqa: BLE001 - the failure is the observation
            res['raised'] = True
            res['error'] = type(e).__name__
    with open(out, 'w') as f:
        json.dump(res, f)
    if scenario != 'dead_peer':
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
