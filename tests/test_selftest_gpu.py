"""Device self-tests: the division fast path over every float, and the error
path of a bounded wait (no GPU fault: the wait gives up and reports)."""
import ctypes

import pytest

from thesis_gb300 import lib as L

pytestmark = pytest.mark.gpu

COEFFS = [4, 6, 8, 12, 16, 18, 24, 32, 36, 48, 64, 96]


@pytest.mark.parametrize("coeff", COEFFS)
def test_division_fast_path_matches_ieee_for_all_floats(cuda, coeff):
    bad = ctypes.c_ulonglong(123)
    first = ctypes.c_uint(0)
    L.check(L.load().stencil_selftest_div(coeff, ctypes.byref(bad), ctypes.byref(first)),
            "stencil_selftest_div")
    assert bad.value == 0, "first mismatching bit pattern 0x%08x" % first.value


def test_selftest_div_rejects_unused_coefficient(cuda):
    bad = ctypes.c_ulonglong()
    assert L.load().stencil_selftest_div(7, ctypes.byref(bad), None) == L.EINVAL


def test_bounded_wait_gives_up_and_reports(cuda):
    from thesis_gb300 import stencil as S
    assert S.device_status() == 0
    done, status = ctypes.c_int(7), ctypes.c_int(0)
    L.check(L.load().stencil_selftest_wait(50, ctypes.byref(done), ctypes.byref(status)),
            "stencil_selftest_wait")
    assert done.value == 0          # the wait did not complete
    assert status.value & 1         # timeout bit set in the device status word
    assert S.device_status() == 0   # cleared by the read; context still usable
    u = S.init_uniform((16, 16, 16), 1)
    assert float(u.sum()) > 0
