"""The GPU harness of the reference's particle kernels (oracle/ref_gpu_harness.cu) takes
its bindings in the layout of the tests' OrcBindings (the CPU harness's record): the
record sizes agree, and the harness reports the reference's launch grid (blocks of 256
threads) for the padding of the per-particle arrays.  No GPU needed."""
import ctypes as C
import os

import pytest

import orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _harness():
    path = os.path.join(ROOT, "oracle", "_ref", "librefgpu_nofma.so")
    if not os.path.exists(path):
        pytest.skip("the reference's kernels are not built here (no decoded sources)")
    return C.CDLL(path)


def test_bindings_layout_matches_the_tests_record():
    g = _harness()
    assert g.refgpu_sizeof_bindings() == C.sizeof(orc.OrcBindings)


@pytest.mark.parametrize("n,grid", [(0, 0), (1, 1), (255, 255), (256, 256), (257, 512), (108186, 108288)])
def test_grid_items_round_up_to_the_reference_block(n, grid):
    assert _harness().refgpu_grid_items(n) == grid
