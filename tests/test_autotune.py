"""The autotuner's choice rule, on the host: candidates are compared by their
best build time, and a build time of zero (stage events that did not record)
stops the tuning instead of picking an arbitrary candidate."""
import pytest

from libqdt_gb300 import autotune as A


def test_best_build_ms_takes_the_minimum():
    times = iter([9.0, 5.0, 4.0, 6.0])
    assert A._best_build_ms(lambda: next(times)) == 4.0


def test_best_build_ms_rejects_zero_times():
    with pytest.raises(RuntimeError):
        A._best_build_ms(lambda: 0.0)
