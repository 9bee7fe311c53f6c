"""Tensor-core operand layouts (TMA 128-byte swizzle, K-major and MN-major
shared-memory descriptors, tensor-memory A operand) on exact integer data, and
the packed (f32x2) double-float exp, add and mul of the exact-slice FP64 form
bitwise against the scalar ones."""
import pytest

pytestmark = pytest.mark.gpu


def test_tensor_core_operand_layouts(pkg):
    errs = pkg.selftest()
    assert errs == [0.0, 0.0, 0.0, 0.0], errs
