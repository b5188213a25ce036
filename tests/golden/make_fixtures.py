"""Generate the committed fixtures under tests/golden/ from the reference tree.

Run in a checkout that has the codec-arena reference mounted (default
/root/reference, or pass its path). The GPU machine does not need the reference:
only the files written here are read at test and bench time.

Fixtures:
  surrogate_v3_161.txt  the reference's committed surrogate (state/surrogate.txt)
  pop_seed_96.txt       the reference's seed population (pop/seed.txt), the
                        default elites of its `make screen` target
  evolve_golden.json    outputs of brain/evolve.py's own Python functions
                        (features, load_weights migration, genome_line,
                        refit_surrogate) on seeded inputs, imported from the
                        reference
"""
from __future__ import annotations

import importlib.util
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    shutil.copyfile(os.path.join(ref, "state", "surrogate.txt"), os.path.join(HERE, "surrogate_v3_161.txt"))
    shutil.copyfile(os.path.join(ref, "pop", "seed.txt"), os.path.join(HERE, "pop_seed_96.txt"))

    spec = importlib.util.spec_from_file_location("ref_evolve", os.path.join(ref, "brain", "evolve.py"))
    ev = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ev)

    rng = np.random.default_rng(20261203)
    genes = rng.random((6, 29)).round(6).tolist()
    out = {"features": [[float(v) for v in ev.features(g)] for g in genes], "genes": genes}
    # load_weights migration of every compact layout
    mig = {}
    tmp = os.path.join(HERE, "_tmp_w.txt")
    for n in (153, 159, 161, 164, 165, 166):
        w = [float(i) for i in range(n)]
        ev.save_weights(tmp, w)
        mig[str(n)] = ev.load_weights(tmp)
    os.remove(tmp)
    out["load_weights"] = mig
    out["genome_line"] = [ev.genome_line({"id": 7, "gen": 3, "pa": 1, "pb": 2, "tribe": 5, "g": g})
                          for g in genes[:3]]
    # ridge refit toward the prior (rows: 400 seeded genomes, quadratic truth + noise)
    rows_g = rng.random((400, 29))
    w_true = rng.normal(0, 1, 166)
    y = np.array([np.dot(ev.features(list(g)), w_true) for g in rows_g]) + rng.normal(0, 0.5, 400)
    prior = rng.normal(0, 0.1, 166).tolist()
    outp = os.path.join(HERE, "_tmp_refit.txt")
    ok = ev.refit_surrogate([(list(g), float(v)) for g, v in zip(rows_g, y)], prior, outp, alpha=50.0)
    out["refit"] = {"rows_genes": rows_g.tolist(), "rows_fit": y.tolist(), "prior": prior, "alpha": 50.0,
                    "written": bool(ok), "weights": ev.load_weights(outp) if ok else None}
    if ok:
        os.remove(outp)
    with open(os.path.join(HERE, "evolve_golden.json"), "w") as f:
        json.dump(out, f)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
