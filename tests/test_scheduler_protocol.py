"""The scheduler-object protocol Finch's compute uses (src/scheduler/
LogicExecutor.jl:71-96): a callable with set_options, and == and hash over
its options, so that equal schedulers share cached programs."""
import pytest

from finchgb import get_scheduler, set_scheduler, with_scheduler
from finchgb.galley import GalleyScheduler, galley_scheduler
from finchgb.scheduler import GB300Scheduler


def test_equal_options_equal_schedulers():
    a, b = GB300Scheduler(), GB300Scheduler()
    assert a == b and hash(a) == hash(b)
    a.last_kernel = "spmv"  # state, not an option
    assert a == b and hash(a) == hash(b)
    assert GB300Scheduler(finch_order=True) != a
    assert galley_scheduler() == galley_scheduler()
    assert galley_scheduler(estimator="uniform") != galley_scheduler()
    assert galley_scheduler() != GB300Scheduler()  # different kinds never compare equal
    cache = {GB300Scheduler(): 1, galley_scheduler(): 2}
    assert cache[GB300Scheduler()] == 1 and cache[galley_scheduler()] == 2


def test_set_options_returns_a_new_scheduler():
    a = GB300Scheduler()
    b = a.set_options(finch_order=True)
    assert b is not a and b.finch_order and not a.finch_order
    assert b == GB300Scheduler(finch_order=True)
    g = galley_scheduler().set_options(estimator="uniform", verbose=True)
    assert isinstance(g, GalleyScheduler) and g.estimator == "uniform" and g.verbose
    with pytest.raises(TypeError):
        a.set_options(no_such_option=1)
    with pytest.raises(ValueError):
        galley_scheduler().set_options(estimator="exact")


def test_with_scheduler_restores_the_previous_one():
    before = get_scheduler()
    s = GB300Scheduler(finch_order=True)
    with with_scheduler(s):
        assert get_scheduler() == s
    assert get_scheduler() is before
    set_scheduler(s)
    try:
        assert get_scheduler() == GB300Scheduler(finch_order=True)
    finally:
        set_scheduler(before)
