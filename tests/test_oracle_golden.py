"""The oracle against the reference itself.

tests/golden/golden.json holds, for each configuration in
tests/golden/configs.py, the digests of every snapshot and the per-step log
numbers that the reference's own sources produced (built for the CPU by
oracle/ref, run by tests/golden/make_golden.py); for the long runs
(configs.LONG_CONFIGS, among them the reference's shipped input with its
example.ini) those of the first configs.FIRST_STEPS steps.  The oracle must
reproduce them: integer state (topology, flags, candidates, lists) bit for bit
everywhere, and the full snapshot text byte for byte on x86-64, where the
fixtures were made (libm's last bit can differ on other CPUs).
"""
import json
import os
import platform

import pytest

import configs
import snapshot

GOLDEN = json.load(open(os.path.join(configs.HERE, "golden.json")))


def run_oracle(O, name, tmp):
    _, _, _, seed, mg = configs.ALL_CONFIGS[name]
    nmax = configs.golden_nmax(name)
    ini = configs.write_ini(os.path.join(tmp, "run.ini"), name, os.path.join(tmp, "unused"), nmax=nmax)
    opt = O.parse_ini(ini)
    opt.min_grains = mg
    o = O.Oracle.from_files(opt)
    o.rng_synthetic(seed)
    log = []

    def on_step(x):
        s = x.s
        log.append({"n": s.n, "two_three": [s.last_two_three[i] for i in range(s.n_two_three_iters)],
                    "n_grains": s.curr_n_grains, "nucl_area": "%.16f" % s.nucleated_area,
                    "nucleated_at": s.vrt_id_candidate if s.ev_nucleations else -1})

    snaps = os.path.join(tmp, "snaps")
    assert o.run(snaps, on_step) == 0
    assert o.s.status == 0
    return log, [snapshot.digests(os.path.join(snaps, f)) for f in sorted(os.listdir(snaps))]


@pytest.mark.parametrize("name", sorted(configs.ALL_CONFIGS))
def test_oracle_reproduces_reference(oracle_mod, name, tmp_path):
    log, snaps = run_oracle(oracle_mod, name, str(tmp_path))
    g = GOLDEN[name]
    assert len(log) == len(g["steps"])
    for mine, ref in zip(log, g["steps"]):
        assert mine == ref, "step %d differs: %s vs %s" % (ref["n"], mine, ref)
    assert len(snaps) == len(g["snapshots"])
    exact_text = platform.machine() == "x86_64"
    for k, ((full, topo), (gfull, gtopo)) in enumerate(zip(snaps, g["snapshots"])):
        assert topo == gtopo, "snapshot %d: integer state differs" % k
        if exact_text:
            assert full == gfull, "snapshot %d: text differs" % k


def test_golden_covers_every_event_kind():
    steps = [s for g in GOLDEN.values() for s in g["steps"]]
    assert any(any(s["two_three"]) for s in GOLDEN["example_ref2k"]["steps"] + GOLDEN["events_m1000"]["steps"])
    assert any(any(s["two_three"]) for s in steps), "no 2x3 removal in the fixtures"
    assert sum(s["nucleated_at"] >= 0 for s in steps) >= 10
    removed = [GOLDEN[k]["steps"][0]["n_grains"] - GOLDEN[k]["steps"][-1]["n_grains"] for k in configs.CONFIGS]
    assert min(removed) > 0
