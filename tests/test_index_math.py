"""Index arithmetic of the kernels, checked on the CPU: host programs under
tests/native/ include the kernels' own headers, replay their partitions of
the work and check every buffer index against its bound. Nothing is
launched; only nvcc is needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'wot_gb300', 'csrc')


def _run(name, tmp_path):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('nvcc not available')
    exe = str(tmp_path / name)
    subprocess.run([nvcc, '-std=c++17', '-I', CSRC, '-o', exe, os.path.join(ROOT, 'tests', 'native', name + '.cu')],
                   check=True, capture_output=True, timeout=300)
    out = subprocess.run([exe], check=False, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith('ok'), out.stdout + out.stderr


def test_tensor_core_partition(tmp_path):
    """lse_tc_kernel's stretches and the merge's partial lookup
    (tc_stretch_begin / tc_cta_of): unique in-bounds slots, complete reads,
    and the number of writers per row tile that the in-kernel finish counts."""
    _run('stretch_check', tmp_path)


def test_tensor_core_operand_layout(tmp_path):
    """Packed tile offsets and the MMA's shared-memory descriptors agree
    (core_offset / smem_desc / idesc_f16_f32 in wotg_tc.cuh)."""
    _run('layout_check', tmp_path)
