"""On the GPU, the integer-pipe double operations give exactly the bits of the FP64 instructions
they replace (random operands of every kind: any bit pattern, integers, wide exponent ranges,
quotients near one and exact quotients), and sin / cos stay within 2 ulp of the library's."""
import pytest

import ralgpu as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0x5EED])
def test_softfp_matches_the_fp64_instructions(seed):
    res = R.softfp_selftest(n=1 << 25, seed=seed)
    bad = {op: v for op, v in res.items() if v[0] != 0}
    assert not bad, {op: (n, hex(a), hex(b)) for op, (n, (a, b)) in bad.items()}
