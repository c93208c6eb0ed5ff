"""p-range sharding through the library on one GPU: each shard window of
rsieve.shard is sieved by its own job, and the merged factor list equals the
whole range sieved at once and the oracle's set (the sharded path across GPUs
runs exactly these calls, one shard per device, with no collective)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3, 8])
def test_shards_through_library_match_whole_range(rs, oracle_mod, world):
    import rsieve.shard as sh
    import rsieve.synth as S

    b, s, ks, nl = S.plain_job(1)
    text = S.to_abcd(b, s, ks, nl)
    p0, p1 = 2**33 + 1, 2**33 + 10**7
    parts = []
    for r in range(world):
        a, z = sh.shard_range(p0, p1, r, world)
        with rs.Job(text, datless=1) as j:
            f, _ = j.sieve(a, z)
        parts.append(f)
    merged = sh.merge(parts)
    with rs.Job(text, datless=1) as j:
        whole, _ = j.sieve(p0, p1)
    key = lambda f: [(int(x["p"]), int(x["k"]), int(x["n"]), int(x["b"]), int(x["c"])) for x in f]
    assert key(merged) == key(whole)
    want, _ = oracle_mod.Job.from_arrays(b, s, ks, [np.asarray(x) for x in nl]).sieve(p0, p1, datless=True)
    assert [x[:3] for x in key(whole)] == [(int(x["p"]), int(x["k"]), int(x["n"])) for x in want]
    assert len(want) >= 50
