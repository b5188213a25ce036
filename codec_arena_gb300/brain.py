"""The screen step of brain/evolve.py, in process, and its file formats.

`screen_generation` replaces the subprocess call at brain/evolve.py:419-454:
it takes the elite dicts evolve.py keeps in memory, runs the GPU screen and
returns promoted dicts (pa, pb, tribe, g) plus the screened count, without
writing elites.txt or reading promoted.txt. With `text_roundtrip=True` the
elites go through the same text the subprocess path uses (genome_line, then
the screen's own parser, including its v6 quirk unless `v6_fix`), and the
promoted genes come back rounded to 4 decimals as evolve.py reads them; the
result then equals the file-based path exactly.

The format helpers mirror evolve.py's own: `load_pop` (:71-101),
`genome_line` (:104-106), `features` (:211-220), `load_weights` (:223-241),
`save_weights` (:244-247); `refit_surrogate` (:250-268) runs on the GPU. The
search-counter bookkeeping mirrors `screens_count.txt` (:621-622) and its
merge in tools/merge_results.py:62-124. `features_full`, `extend_to_full` and
the 465-coefficient weights that screen_generation / refit_surrogate accept
are the full quadratic surface (all 29 genes), which the reference queues in
docs/RESEARCH_V05C.md:99-102 but does not implement.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import genome as _genome
from . import parallel as _parallel
from . import screen as _screen
from ._lib import GENOME_DTYPE

NG_EFF, NR_REG = 23, 6
NG = NG_EFF + NR_REG
REG_DEFAULT = 0.5
NEW_GENE_DEFAULT = 0.0
N_NEW = 7


def load_pop(path: str) -> List[Dict]:
    """brain/evolve.py:71-101: pop lines of 21/27/29/32/33/34 tokens migrated
    to 34 tokens (5 + 29 genes); other widths are skipped."""
    pop = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            t = line.split()
            if len(t) == 5 + 16:
                t = t + [str(NEW_GENE_DEFAULT)] * N_NEW + [str(REG_DEFAULT)] * NR_REG
            elif len(t) == 5 + 22:
                t = t[: 5 + 16] + [str(NEW_GENE_DEFAULT)] * N_NEW + t[5 + 16:]
            elif len(t) == 5 + 24:
                t = t[: 5 + 18] + [str(NEW_GENE_DEFAULT)] * 5 + t[5 + 18:]
            elif len(t) == 5 + 27:
                t = t[: 5 + 21] + [str(NEW_GENE_DEFAULT)] * 2 + t[5 + 21:]
            elif len(t) == 5 + 28:
                t = t[: 5 + 22] + [str(NEW_GENE_DEFAULT)] + t[5 + 22:]
            if len(t) != 5 + NG:
                continue
            pop.append({"id": int(t[0]), "gen": int(t[1]), "pa": int(t[2]), "pb": int(t[3]),
                        "tribe": int(t[4]), "g": [float(x) for x in t[5:]]})
    return pop


def genome_line(g: Dict) -> str:
    """brain/evolve.py:104-106."""
    return f"{g['id']} {g['gen']} {g['pa']} {g['pb']} {g['tribe']} " + " ".join(f"{x:.4f}" for x in g["g"])


def features(genes) -> np.ndarray:
    """brain/evolve.py:211-220, vectorised: (n, 29) genes -> (n, 166) features
    [1 | 29 linear | g_i g_j for j <= i < 16]."""
    g = np.atleast_2d(np.asarray(genes, dtype=np.float64))
    ii, jj = np.tril_indices(16)  # row-major: i outer, j <= i inner
    quad = g[:, ii] * g[:, jj]
    return np.concatenate([np.ones((g.shape[0], 1)), g, quad], axis=1)


FULL_NF = 465  # the full surface: all 29 genes quadratic (csx_screen.h)


def features_full(genes) -> np.ndarray:
    """The full surface's features: (n, 29) genes -> (n, 465)
    [1 | 29 linear | g_i g_j for j <= i < 29], the pattern of features()
    with the quadratic block over every gene (the extension
    docs/RESEARCH_V05C.md:99-102 queues; no reference code)."""
    g = np.atleast_2d(np.asarray(genes, dtype=np.float64))
    ii, jj = np.tril_indices(29)
    return np.concatenate([np.ones((g.shape[0], 1)), g, g[:, ii] * g[:, jj]], axis=1)


def extend_to_full(w: Sequence[float]) -> List[float]:
    """A 166-coefficient model (any layout after load_weights) as the same
    surface in the full layout: the quadratic block over genes 0..15 placed in
    the 29-gene triangle, the new pairs 0, and the intercept times 16 (the
    reference's Model.score counts w0 in each of its 16 lanes)."""
    w = [float(x) for x in w]
    if len(w) != 166:
        raise ValueError("extend_to_full takes the 166-coefficient layout")
    full = [16.0 * w[0]] + w[1:30]
    q = 30
    for i in range(29):
        for j in range(i + 1):
            full.append(w[q] if i < 16 else 0.0)
            q += 1 if i < 16 else 0
    return full


def load_weights(path: str) -> List[float]:
    """brain/evolve.py:223-241: any compact layout migrated to 166. A file of
    465 coefficients holds the full surface and is returned as it is."""
    with open(path) as f:
        toks = f.read().split()
    n = int(toks[0])
    return migrate_weights([float(x) for x in toks[1:1 + n]])


def migrate_weights(w: Sequence[float]) -> List[float]:
    """load_weights' migration of a compact weight list (brain/evolve.py:228-240)."""
    w = [float(x) for x in w]
    n = len(w)
    if n == 153:
        w = w[:17] + [0.0] * 13 + w[17:]
    elif n == 159:
        w = w[:17] + [0.0] * 7 + w[17:]
    elif n == 161:
        w = w[:19] + [0.0] * 5 + w[19:]
    elif n == 164:
        w = w[:22] + [0.0] * 2 + w[22:]
    elif n == 165:
        w = w[:29] + [0.0] + w[29:]
    return w


def save_weights(path: str, w: Sequence[float]) -> None:
    """brain/evolve.py:244-247."""
    with open(path, "w") as f:
        f.write(f"{len(w)}\n")
        f.write(" ".join(f"{x:.8e}" for x in w) + "\n")


def elites_array(elites: Sequence[Dict], text_roundtrip: bool = False, v6_fix: bool = False) -> np.ndarray:
    """Elite dicts -> GENOME_DTYPE records, directly or through elites.txt text."""
    if text_roundtrip:
        return _genome.load_elites_text("".join(genome_line(g) + "\n" for g in elites), v6_fix=v6_fix)
    out = np.zeros(len(elites), dtype=GENOME_DTYPE)
    for i, g in enumerate(elites):
        out[i]["id"], out[i]["gen"], out[i]["pa"], out[i]["pb"], out[i]["tribe"] = (
            g["id"], g["gen"], g["pa"], g["pb"], g["tribe"])
        out[i]["g"] = np.asarray(g["g"], dtype=np.float32)
    return out


def screen_generation(elites: Sequence[Dict], model, *, screens: int, keep: int, seed: int, shard: int,
                      gen: int, threads: int = 4, sigma_decay: float = 0.93, jump: float = 0.02,
                      imm: float = 0.01, text_roundtrip: bool = False,
                      v6_fix: bool = False) -> Tuple[List[Dict], int]:
    """One generation's screen as brain/evolve.py:431-454 runs it, in process.

    `model` is a screen.Model, a screen.ModelFull or compact weights (465 of
    them: the full surface). Returns (promoted, screened): promoted dicts
    carry pa, pb, tribe and the 29 genes, best first.
    """
    if not isinstance(model, (_screen.Model, _screen.ModelFull)):
        w = np.asarray(model, dtype=np.float32)
        model = _screen.ModelFull.from_compact(w) if w.shape[0] == FULL_NF else _screen.Model.from_compact(w)
    sigma = 0.12 * (sigma_decay ** gen)
    if text_roundtrip:  # evolve.py passes sigma as "%.4f" text
        sigma = float(f"{sigma:.4f}")
    cfg = _screen.Cfg(int(screens), int(keep), _parallel.island_seed(seed, shard, gen), threads=int(threads),
                      sigma=sigma, jump_p=jump, imm_p=imm)
    surv, screened = _screen.screen(cfg, model, elites_array(elites, text_roundtrip, v6_fix))
    promoted = []
    for r in surv:
        g = [float(x) for x in r["g"]]
        if text_roundtrip:
            g = [float(f"{x:.4f}") for x in g]
        promoted.append({"id": 0, "gen": 0, "pa": int(r["pa"]), "pb": int(r["pb"]), "tribe": int(r["tribe"]),
                         "g": g})
    return promoted, screened


def refit_surrogate(rows, prior_w: Sequence[float], out_path: str, alpha: float = 50.0) -> bool:
    """brain/evolve.py:250-268 on the GPU: ridge refit toward the prior,
    min ||Xw - y||² + α||w - w_prior||², normal equations and Cholesky in
    FP64. rows: (genes, fit) pairs. As the reference: False (nothing written)
    below 300 rows or when the prior's length is not the feature count; here
    the prior may also hold the full surface's 465 coefficients."""
    import torch

    from . import surrogate as _sg

    if len(rows) < 300:
        return False
    prior = np.asarray(prior_w, dtype=np.float64)
    if prior.shape[0] not in (166, FULL_NF):
        return False
    genes = torch.tensor(np.array([list(g) for g, _ in rows], dtype=np.float32), device="cuda")
    fit = torch.tensor(np.array([f for _, f in rows], dtype=np.float64), device="cuda")
    if genes.shape[1] != 29:
        return False
    w = _sg.refit(genes, fit, torch.from_numpy(prior).cuda(), alpha=alpha)
    save_weights(out_path, [float(v) for v in w.cpu().numpy()])
    return True


def next_population(elites: Sequence[Dict], promoted: Sequence[Dict], *, shard: int, gen: int, pop: int,
                    keep: int) -> List[Dict]:
    """brain/evolve.py:455-461: elites first, then up to `keep` promoted genomes
    with the ids and generation evolve.py assigns. The caller tops the list up
    to `pop` with its own tournament breeding (:462-474)."""
    nxt = [dict(g) for g in elites]
    for p in list(promoted)[:keep]:
        nxt.append({"id": shard * 10_000_000 + gen * pop + len(nxt), "gen": gen + 1, "pa": p["pa"],
                    "pb": p["pb"], "tribe": p["tribe"], "g": list(p["g"])})
    return nxt


def write_screens_count(out_dir: str, n_screens: int) -> str:
    """brain/evolve.py:621-622: a shard's search counter file."""
    import os

    path = os.path.join(out_dir, "screens_count.txt")
    with open(path, "w") as f:
        f.write(str(int(n_screens)))
    return path


_EVAL_MILESTONES = [("1e5", 100_000), ("1e6", 1_000_000), ("1e7", 10_000_000), ("1e8", 100_000_000),
                    ("1e9", 1_000_000_000)]
_SEARCH_MILESTONES = [("1e6", 1_000_000), ("1e9", 1_000_000_000), ("1e12", 1_000_000_000_000)]


def update_lifetime_counters(in_dir: str, state: Dict) -> Dict:
    """The counter part of tools/merge_results.py:62-124: sum every shard's
    evals_count.txt and screens_count.txt (shard-* directories of `in_dir`)
    into `state` (lifetime_evals, search_evals = evals + screens, runs,
    milestones); returns the updated copy."""
    import glob
    import os

    n_evals = n_screens = 0
    for sd in sorted(glob.glob(os.path.join(in_dir, "shard-*"))):
        for name in ("evals_count.txt", "screens_count.txt"):
            p = os.path.join(sd, name)
            if os.path.exists(p):
                with open(p) as f:
                    v = int(f.read().strip() or 0)
                if name == "evals_count.txt":
                    n_evals += v
                else:
                    n_screens += v
    st = dict(state) if state else {"lifetime_evals": 0, "runs": 0, "milestones": {}}
    st.setdefault("search_evals", st.get("lifetime_evals", 0))
    st["lifetime_evals"] = st.get("lifetime_evals", 0) + n_evals
    st["search_evals"] += n_evals + n_screens
    st["runs"] = st.get("runs", 0) + 1
    st["milestones"] = dict(st.get("milestones", {}))
    st["search_milestones"] = dict(st.get("search_milestones", {}))
    for m, key in _EVAL_MILESTONES:
        if st["lifetime_evals"] >= key and m not in st["milestones"]:
            st["milestones"][m] = f"run {st['runs']}"
    for m, key in _SEARCH_MILESTONES:
        if st["search_evals"] >= key and m not in st["search_milestones"]:
            st["search_milestones"][m] = f"run {st['runs']}"
    return st


__all__ = ["load_pop", "genome_line", "features", "load_weights", "save_weights", "elites_array",
           "screen_generation", "next_population", "write_screens_count", "update_lifetime_counters"]
