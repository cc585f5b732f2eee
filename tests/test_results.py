"""Result lines in the schema of micrographia's bench/results.jsonl (the field order of
crates/bench/src/main.rs:262-277), plus this engine's extra figures after them."""

import json

import pytest

from micrographia_gb300 import results

REFERENCE_FIELDS = ["time", "commit", "device", "engine", "mode", "order", "dim", "pair", "density", "n", "steps_per_s",
                    "ns_per_particle_step", "phase_ns", "copy_gbps"]


def test_record_has_the_reference_fields_in_order(tmp_path):
    r = results.record(engine="gb300-int-f32", mode="verlet", order="lattice", dim=3, pair="lj", density=0.8442, n=1048576,
                       steps_per_s=2650.55, phase_ns={"force": 251000.4, "rebuild": 105000}, copy_gbps=6787.62, commit="abc123",
                       device="GB300 (CUDA)", when=1792473954, atom_steps_per_s=2.78e9, p99_ms=125.0)
    assert list(r)[: len(REFERENCE_FIELDS)] == REFERENCE_FIELDS
    assert list(r)[len(REFERENCE_FIELDS):] == ["atom_steps_per_s", "p99_ms"]
    assert r["steps_per_s"] == 2650.6 and r["ns_per_particle_step"] == round(1e9 / (2650.55 * 1048576), 3)
    assert r["phase_ns"] == {"force": 251000, "rebuild": 105000}
    path = tmp_path / "results.jsonl"
    results.append(path, [r, r])
    lines = path.read_text().splitlines()
    assert len(lines) == 2 and json.loads(lines[0]) == r


def test_unknown_fields_are_refused():
    with pytest.raises(ValueError):
        results.record(engine="e", mode="m", order="o", dim=2, pair="lj", density=0.7, n=10, steps_per_s=1.0, phase_ns={},
                       copy_gbps=1.0, bogus=1)
