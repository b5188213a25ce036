"""The pruning screen's bound, restated in float64 and checked on the
oracle's candidates (CPU, no GPU).

The GPU screen skips a crossover candidate when an upper bound of its score,
taken from its parents and crossover bits before the mutation draws, is below
the K-th score. The bound's claim is that for every crossover candidate

    f(final genes) <= f(y) + s * sum_k |grad_k f(y)| + c0 + c_jump,

with y_k = clamp01(parent gene chosen by the crossover bit), s = min(|sigma| +
2^-24, 1), c0 = s * sum_{k>=16} |w_k| + s^2 * (sum_i max(Q_ii, 0) +
sum_{j<i} |Q_ij|) and c_jump the per-gene jump bound (0 without a jump).
Here the crossover bits come from splitmix64 in numpy at each candidate's
draw positions, the final genes from the oracle's candidate dump, and f in
float64. The f32 rounding margins are the GPU tests' business.
"""
import numpy as np
import pytest

G = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def mix(states):
    with np.errstate(over="ignore"):
        z = states
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def draw(seed_t, pos):
    """Output of draw `pos` (0-based) of the stream seeded seed_t."""
    with np.errstate(over="ignore"):
        return mix(np.uint64(seed_t) + (pos.astype(np.uint64) + np.uint64(1)) * G)


def stream_seed(seed, t):
    with np.errstate(over="ignore"):
        return np.uint64(seed) ^ (G * np.uint64(t + 1))


def model_arrays(orc, w):
    m = orc.model_from_compact(w)
    wl = np.array(m.w_lin[:], dtype=np.float64)
    Q = np.tril(np.array(m.w_quad[:], dtype=np.float64).reshape(16, 16))
    return float(m.w0), wl, Q


def surface(w0, wl, Q, g):
    return 16.0 * w0 + g @ wl + np.einsum("ni,ij,nj->n", g[:, :16], Q, g[:, :16])


def jump_bound(wl, Q):
    c = np.zeros(29)
    for j in range(29):
        a_hi = a_lo = wl[j]
        qjj = 0.0
        if j < 16:
            for i in range(16):
                q = Q[j, i] if i <= j else Q[i, j]
                if i == j:
                    qjj = q
                elif q > 0:
                    a_hi += q
                else:
                    a_lo += q
        c[j] = max(max(0.0, a_hi) + max(0.0, qjj), max(0.0, -a_lo) + max(0.0, -qjj))
    return c


def bound(w0, wl, Q, y, sigma):
    s = min(abs(float(sigma)) + 2.0 ** -24, 1.0)
    Qs = Q + Q.T
    grad = np.tile(wl, (len(y), 1))
    grad[:, :16] += y[:, :16] @ Qs.T
    qpos = np.maximum(np.diag(Q), 0).sum() + np.abs(np.tril(Q, -1)).sum()
    c0 = s * np.abs(wl[16:]).sum() + s * s * qpos
    return surface(w0, wl, Q, y) + s * np.abs(grad).sum(1) + c0


def check_stream(orc, w, el, sigma, imm, jump, t, n, seed=7):
    c = orc.cfg(10**9, 1, seed, threads=8, sigma=sigma, jump_p=jump, imm_p=imm)
    cand = orc.stream_dump(c, orc.model_from_compact(w), el, t, n)
    w0, wl, Q = model_arrays(orc, w)
    st = stream_seed(seed, t)
    p = cand["draw"].astype(np.uint64)
    imm_thr = np.ceil(np.float64(np.float32(imm)) * 2**24) if imm > 0 else 0
    is_imm = (draw(st, p + np.uint64(2)) >> np.uint64(40)).astype(np.float64) < imm_thr
    # parents: (next() >> 32) % ne for draws p and p + 1
    ne = len(el)
    ea = ((draw(st, p) >> np.uint64(32)) % np.uint64(ne)).astype(np.int64)
    eb = ((draw(st, p + np.uint64(1)) >> np.uint64(32)) % np.uint64(ne)).astype(np.int64)
    assert np.array_equal(el["id"][ea], cand["pa"]) and np.array_equal(el["id"][eb], cand["pb"])
    k = np.arange(29, dtype=np.uint64)
    bits = (draw(st, p[:, None] + np.uint64(3) + np.uint64(2) * k[None, :]) & np.uint64(1)).astype(bool)
    eg = el["g"].astype(np.float64)
    eg = np.where(np.isnan(eg), np.inf, eg)
    y = np.clip(np.where(bits, eg[eb], eg[ea]), 0.0, 1.0)
    b = bound(w0, wl, Q, y, sigma)
    # the jump: index at draw p + 62 for crossover candidates that jump
    jthr = np.ceil(np.float64(np.float32(jump)) * 2**24) if jump > 0 else 0
    jumps = (draw(st, p + np.uint64(61)) >> np.uint64(40)).astype(np.float64) < jthr
    jidx = ((draw(st, p + np.uint64(62)) >> np.uint64(32)) % np.uint64(29)).astype(np.int64)
    cj = np.where(jumps, jump_bound(wl, Q)[jidx], 0.0)
    f = surface(w0, wl, Q, cand["g"].astype(np.float64))
    xo = ~is_imm
    assert xo.sum() > 0
    slack = 1e-9 * (16 * abs(w0) + np.abs(wl).sum() + np.abs(Q).sum())
    viol = f[xo] - (b[xo] + cj[xo])
    assert np.all(viol <= slack), f"bound violated by {viol.max()}"
    return b[xo] + cj[xo] - f[xo]


MODELS = {
    "v3_committed": lambda wl_: wl_.surrogate_161(),
    "v1_normal": lambda wl_: wl_.seeded_normal_model(seed=2),
    "v6_random_tail": lambda wl_: np.random.default_rng(5).normal(0, 3, 166).astype(np.float32),
}


@pytest.mark.parametrize("name", sorted(MODELS))
@pytest.mark.parametrize("sigma", [0.12, 0.5, 0.0, 1e-30, 2.0, -0.25])
def test_bound_holds_on_oracle_candidates(orc, name, sigma):
    from codec_arena_gb300 import workloads as wl_

    w = MODELS[name](wl_)
    el = wl_.seeded_elites(64)
    gap = check_stream(orc, w, el, sigma, 0.01, 0.3, t=1, n=20_000)
    assert gap.min() >= 0.0 or gap.min() > -1e-6


def test_bound_with_extreme_elite_genes(orc):
    """Parent genes outside [0, 1], +-inf and NaN: y clamps them, and the
    mutated gene stays within s of y."""
    from codec_arena_gb300 import workloads as wl_

    el = wl_.seeded_elites(12)
    el["g"][0, :5] = [-0.0, -3.0, 7.5, np.inf, -np.inf]
    el["g"][1, :3] = [np.nan, 1.0, 0.0]
    el["g"][2, :16] = np.linspace(-0.2, 1.2, 16)
    for sigma in (0.12, 0.9):
        check_stream(orc, wl_.surrogate_161(), el, sigma, 0.0, 0.5, t=0, n=20_000)


def test_bound_is_tight_enough_to_prune(orc):
    """On the bench workload's surface the bound is typically within a few
    score units of the real value (the prune rate depends on it)."""
    from codec_arena_gb300 import workloads as wl_

    gap = check_stream(orc, wl_.surrogate_161(), wl_.seeded_elites(64), 0.12, 0.01, 0.02, t=0, n=20_000)
    assert np.median(gap) < 60.0
