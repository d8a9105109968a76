"""fgb_gather_ceiling: the random-gather rate the row-gathering kernels are
read against.  It must report a finite positive rate, serve an L2-sized
working set at least as fast as one far larger than L2, and reject widths
outside its list."""
import pytest

from finchgb import _lib as L
from finchgb import device as dev

pytestmark = pytest.mark.gpu


def test_gather_ceiling_orders_working_sets():
    small = dev.gather_ceiling(16 << 20, 128, gathers=1 << 22)
    large = dev.gather_ceiling(1 << 30, 128, gathers=1 << 22)
    assert 0 < large and 0 < small
    assert small > 0.9 * large


@pytest.mark.parametrize("width", [4, 8, 16, 64, 512])
def test_gather_ceiling_widths(width):
    assert dev.gather_ceiling(64 << 20, width, gathers=1 << 20) > 0


@pytest.mark.parametrize("width,ws,gathers", [(24, 1 << 20, 1024), (1024, 1 << 20, 1024), (2, 1 << 20, 1024),
                                              (128, 1024, 1024), (128, 1 << 20, 0)])
def test_gather_ceiling_rejects(width, ws, gathers):
    with pytest.raises(L.FinchGBError) as e:
        dev.gather_ceiling(ws, width, gathers=gathers)
    assert e.value.status == L.EINVAL
