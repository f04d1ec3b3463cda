"""CPU: the work models bench.py divides by (algorithmic flops and bytes per
cell, FP64-pipe instructions of the plain and even-odd kernels), checked
against hand counts and the reference's conventions."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_models", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_flops_and_bytes_per_cell(bench):
    # mass 4Qn(n^2+Qn+Q^2)+Q^3, stiffness 4Qn(2n^2+3Qn+3Q^2)+15Q^3; bytes s(2n^3 + c Q^3)
    assert bench.flops_per_cell(0, 4, 5) == 5005
    assert bench.flops_per_cell(1, 5, 6) == 33000
    assert bench.flops_per_cell(1, 7, 8) == 110272
    assert bench.bytes_per_cell(0, 4, 5, 8) == 2024
    assert bench.bytes_per_cell(1, 5, 6, 8) == 12368
    assert bench.bytes_per_cell(1, 5, 6, 4) == 6184
    # affine: one factor set per cell
    assert bench.bytes_per_cell(1, 5, 6, 8, affine=True) == 8 * (250 + 6)
    assert bench.bytes_per_cell(0, 4, 5, 4, affine=True) == 4 * (128 + 1)


def test_reference_convention_at_q_equal_n(bench):
    # bench_mass.cpp:122 counts 6(2n^4+n^3) at Q = n; the convention here
    # counts Q^3 multiplies where the reference counts n^3 twice
    n = 4
    assert bench.flops_per_cell(0, n, n) == 4 * n * n * 3 * n * n + n ** 3


def test_pipe_instruction_model(bench):
    # plain: one FMA per multiply-add plus the point-wise work
    assert bench.pipe_instr_per_cell(1, 5, 6, False) == 16824
    assert bench.pipe_instr_per_cell(1, 5, 6, True) == 14294
    # even-odd issues fewer instructions at every degree of the workloads
    for op, n, q in ((0, 4, 5), (1, 5, 6), (1, 7, 8), (0, 8, 9)):
        assert bench.pipe_instr_per_cell(op, n, q, True) < bench.pipe_instr_per_cell(op, n, q, False)
    # affine mass scales N inputs per pencil instead of Q points
    d = bench.pipe_instr_per_cell(0, 4, 5, False) - bench.pipe_instr_per_cell(0, 4, 5, False, True)
    assert d == 5 ** 3 - 4 ** 3
    # stiffness: the point-wise 9 per point is the same with or without affine geometry
    assert bench.pipe_instr_per_cell(1, 5, 6, True, True) == bench.pipe_instr_per_cell(1, 5, 6, True)


def test_even_odd_flops_below_convention(bench):
    for op, n, q in ((0, 4, 5), (1, 5, 6), (1, 7, 8)):
        assert bench.flops_per_cell_even_odd(op, n, q) < bench.flops_per_cell(op, n, q)
