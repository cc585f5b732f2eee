"""The self-check module (crates/md/src/checks.rs): its SplitMix64 on the CPU, every named check
on the GPU."""

import numpy as np
import pytest

from micrographia_gb300 import checks


def test_splitmix_known_answers():
    """SplitMix64 from seed 0 starts 0xE220A8397B1DCDAF (the generator's published first output);
    a numpy uint64 restatement agrees over 1000 draws from seed 4 (the permutation check's)."""
    assert checks.SplitMix(0).next_u64() == 0xE220A8397B1DCDAF
    r = checks.SplitMix(4)
    s = np.uint64(4)
    with np.errstate(over="ignore"):
        for _ in range(1000):
            s = s + np.uint64(0x9E3779B97F4A7C15)
            z = s
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            assert r.next_u64() == int(z ^ (z >> np.uint64(31)))


def test_unknown_check_is_an_error():
    ok, msg = checks.run("md_nonsense")
    assert not ok and "unknown check" in msg


@pytest.mark.gpu
@pytest.mark.parametrize("name", checks.NAMES)
def test_every_check_passes_on_the_gpu(name):
    """checks::run for each of checks::NAMES (checks.rs:10)."""
    ok, msg = checks.run(name)
    assert ok, msg
