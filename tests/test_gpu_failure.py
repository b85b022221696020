"""Failure detection without a GPU fault: a look-back wait on a status word that nothing writes
ends at its bound with RAL_ERROR_TIMEOUT, and the context keeps working."""
import time

import pytest

import ralgpu as R

pytestmark = pytest.mark.gpu


def test_bounded_lookback_wait_reports_a_timeout_and_the_context_survives():
    t0 = time.time()
    status, kept = R.debug_lookback_timeout(3 * 4096)
    elapsed = time.time() - t0
    assert status == 6                      # RAL_ERROR_TIMEOUT
    assert kept == 3 * 4096                 # the normal run right after
    assert elapsed < 60
