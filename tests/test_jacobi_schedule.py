"""The Jacobi eigen-solver spreads each problem's rows over the CTAs of a
thread-block cluster and passes rows between neighbours as the round-robin
schedule advances. The hand-over logic (tree-embedding_gb300/csrc/
jacobi_sched.h) is host/device code; this compiles it for the host and checks
it against the schedule for every even size up to 260 and 1-16 CTAs."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, '..', 'tree-embedding_gb300', 'csrc')


def test_row_handover_follows_schedule():
    cxx = shutil.which('g++') or shutil.which('c++')
    if cxx is None:
        pytest.skip('no host C++ compiler')
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, 'jacobi_schedule_check')
        subprocess.run([cxx, '-O1', '-std=c++17', '-I', CSRC,
                        os.path.join(HERE, 'native', 'jacobi_schedule_check.cpp'), '-o', exe],
                       check=True)
        out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert 'mismatches 0' in out.stdout
