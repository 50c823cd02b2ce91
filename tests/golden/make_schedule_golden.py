"""Generates schedule.json: the op lists of the reference's own algorithm
manager (MasterSPP/S_SPI_SPRING spring/alg_manager.py, imported from the
reference checkout) for the settings MPR.InitIA builds (spring/mpr.py:110-140)
over whole generation ranges.

    python tests/golden/make_schedule_golden.py
"""
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.refroot import reference_root  # noqa: E402

REF = str(reference_root() / "spring" / "alg_manager.py")

CASES = [
    # alg, it, beta, it_ER, it_eval, it_stab, sigma, threshold, repetitions, decay_exp, start, end, generations
    ("HIO", 40, 0.95, 40, 40, 0, 2.5, 0.03, 3, 1.5, 0.1, 0.95, 100),
    ("RAAR", 100, 0.87, 20, 30, 10, 2.0, 0.05, 4, 1.0, 0.0, 1.0, 10),
    ("HIO", 25, 0.9, 10, 15, 5, 3.0, 0.1, 1, 2.0, 0.3, 0.6, 20),
]


def main():
    spec = importlib.util.spec_from_file_location("ref_alg_manager", REF)
    am = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(am)
    out = []
    for (alg, it, beta, it_er, it_eval, it_stab, sigma, thr, rep, dexp, ds, de, gens) in CASES:
        main_algs = [(am.HIO if alg == "HIO" else am.RAAR)(it, 0, beta, decay_exp=dexp),
                     am.ER(it_er, it_er + it, decay_exp=dexp)]
        stab = [am.ER(it_stab)] if it_stab > 0 else []
        man = am.AlgManager(main=main_algs, stabilization=stab, evaluation=[am.ER(it_eval)], sw_sigma=sigma,
                            sw_threshold=thr, repetitions=rep, scalingstart=int(np.round(ds * gens)),
                            scalingend=int(np.round(de * gens)))
        seqs = []
        for g in range(0, gens + 1):
            area = [1000 + 7 * g, 1500 - 3 * g]
            conv = lambda seq: [[name, [float(p) for p in params]] for name, params in seq]
            seqs.append({"generation": g, "sequence": conv(man.get_sequence(g, area=area)),
                         "first": conv(man.get_sequence(g, area=area, update_support_first=True)),
                         "refine": conv(man.get_sequence(g, area=area, update_support=False)),
                         "support_params": [float(p) for p in man.get_support_params(g)]})
        out.append({"case": [alg, it, beta, it_er, it_eval, it_stab, sigma, thr, rep, dexp, ds, de, gens],
                    "generations": seqs})
    with open(os.path.join(HERE, "schedule.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()
