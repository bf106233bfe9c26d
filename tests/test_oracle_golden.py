"""The C restatement (oracle/lak_oracle.c) reproduces the reference's own
kernel outputs bit for bit on every committed fixture."""
import numpy as np
import pytest

import golden_cases as gc

FIXTURES = gc.load_gram_fixtures()


@pytest.mark.parametrize("fx", FIXTURES, ids=[f.name for f in FIXTURES])
def test_oracle_matches_reference_fixtures(oracle_lib, fx):
    keys = gc.all_keys(fx)
    assert keys
    for key in keys:
        want = fx.expected(key)
        got = gc.run_key("oracle", fx, key)
        assert got.shape == want.shape, key
        # bit-exact: compare the IEEE bit patterns
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (fx.name, key)


def test_fixture_coverage():
    kinds = set()
    for fx in FIXTURES:
        for k in gc.all_keys(fx):
            kinds.add(k.split("/")[0])
    assert kinds == {"AnZt", "AnAt", "An_v", "An_ajdk"}
    assert len(FIXTURES) >= 20
