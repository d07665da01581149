"""Divide-free helpers of the meshlet phases, which must give the same bits as the
IEEE divisions they replace (every value of the path is compared bit for bit with
the oracle):

- the triangle centre's division by 3 (Triangle.RecalculateCenter, mesh.go:1980-1982):
  a multiply by RN(1/3) and one FMA correction, checked for every 32-bit pattern;
- the bucket-sort bin of a depth key (sortingTriangles.go:42-58): a multiply by the
  range's reciprocal with one correction, and the exact division for keys next to a
  bin edge, checked on 4096 seeded ranges x 65536 keys (half of them within a few
  ulps of a bin edge), in both walk orders."""
import ctypes as C

import pytest

from tetra3d_gb300 import abi

pytestmark = pytest.mark.gpu


def test_div3_equals_ieee_division_for_every_float(ctx):
    fn = abi.load().t3d_check_div3
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    bad, first = C.c_uint64(), C.c_uint32()
    assert fn(C.byref(bad), C.byref(first)) == 0
    assert bad.value == 0, f"{bad.value} patterns differ, first 0x{first.value:08x}"


@pytest.mark.parametrize("seed", [1, 2])
def test_fast_bins_equal_divided_bins(ctx, seed):
    fn = abi.load().t3d_check_bins
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint64, C.c_uint32, C.POINTER(C.c_uint64)]
    bad = C.c_uint64()
    assert fn(seed, 65536, C.byref(bad)) == 0
    assert bad.value == 0, f"{bad.value} keys binned differently"
