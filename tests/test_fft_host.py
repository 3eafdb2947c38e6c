"""Host-side check of the Stockham line transform (tests/fft_host_check.cu)
against a direct DFT for every compiled schedule.  CPU only; needs nvcc."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which('nvcc') is None and not os.path.exists('/usr/local/cuda/bin/nvcc'), reason='nvcc absent')
def test_line_fft_schedules(tmp_path):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    exe = str(tmp_path / 'fft_host_check')
    subprocess.run([nvcc, '-std=c++17', '-O2', '-x', 'cu', '-I', os.path.join(ROOT, 'namsa_gb300', 'csrc'),
                    os.path.join(HERE, 'fft_host_check.cu'), '-o', exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count('rel err') >= 11
