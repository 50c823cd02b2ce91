"""The memetic loop's algorithm schedule against the reference's own
algorithm manager (fixture tests/golden/schedule.json, made by
tests/golden/make_schedule_golden.py from spring/alg_manager.py)."""
import json
import os

import pytest

from s_spi_spring_gb300.memetic import MemeticSettings

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "schedule.json")))


def _norm(seq):
    return [[name, [float(p) for p in params]] for name, params in seq]


@pytest.mark.parametrize("k", range(len(GOLD)))
def test_schedule_matches_reference(k):
    alg, it, beta, it_er, it_eval, it_stab, sigma, thr, rep, dexp, ds, de, gens = GOLD[k]["case"]
    s = MemeticSettings(generations=gens, alg=alg, it=it, beta=beta, it_ER=it_er, it_eval=it_eval, it_stab=it_stab,
                        sigma=sigma, threshold=thr, repetitions=rep, decay_exp=dexp, decay_start=ds, decay_end=de)
    man = s.schedule()
    for g in GOLD[k]["generations"]:
        gen = g["generation"]
        area = [1000 + 7 * gen, 1500 - 3 * gen]
        assert _norm(man.sequence(gen, area=area)) == g["sequence"]
        assert _norm(man.sequence(gen, area=area, update_support_first=True)) == g["first"]
        assert _norm(man.sequence(gen, area=area, update_support=False)) == g["refine"]
        assert [float(p) for p in man.support_params(gen)] == g["support_params"]


def test_solver_parses_every_scheduled_op():
    from s_spi_spring_gb300.phase_retrieval import parse_algorithm
    man = MemeticSettings(generations=10).schedule()
    for gen in range(11):
        for name, params in man.sequence(gen, area=[500, 700]):
            assert parse_algorithm(name, params) is not None
