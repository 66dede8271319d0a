"""The batching path (randblas_gb300.batched): many left dense sketches of uneven shapes in one
persistent launch.

1. Every problem of a mixed batch (tails in every dimension, submatrix offsets, Gaussian and
   uniform operators, alpha / beta, alpha = 0, long K that gets split, every tile width,
   Gaussian column tiles taken in cluster pairs, with and without a last odd tile) matches the
   plain single-problem sketch to FP32 accuracy, and a few match the oracle.
2. Results are bitwise reproducible across runs, and equal between the one-shot call, the
   plan and a replayed CUDA graph of the plan.
3. The 512-problem batch with the distribution of the batching benchmark (m log-uniform in
   [2^12, 2^18], n uniform in [16, 512], d = 4n, chained states): sampled problems match the
   plain path.
"""
import numpy as np
import pytest

from gpu_helpers import to_host

pytestmark = pytest.mark.gpu

# d, n, m, ro_s, co_s, family, alpha, beta, tile_config
SHAPES = [
    (64, 16, 5000, 0, 0, 0, 1.0, 0.0, 0),
    (50, 17, 3001, 2, 5, 1, 1.0, 0.0, 3),
    (300, 130, 20000, 0, 0, 0, 0.5, 0.0, 1),
    (128, 64, 60000, 1, 0, 1, 1.0, 1.5, 2),
    (200, 33, 777, 0, 3, 0, -1.0, 0.0, 0),
    (1000, 250, 4096, 0, 0, 1, 1.0, 0.0, 4),
    (96, 512, 150000, 0, 0, 0, 1.0, 0.0, 0),
    (20, 40, 100, 0, 0, 0, 0.0, 2.0, 0),
    (129, 65, 33, 4, 4, 1, 1.0, -0.5, 2),
    (256, 100, 262144, 0, 0, 0, 1.0, 0.0, 0),
    # Gaussian over three column tiles of a 4-aligned submatrix: a cluster pair sharing the
    # operator tiles of interior row blocks, a last odd column tile on its own, a partial row
    # block
    (257, 300, 9000, 3, 8, 0, 1.0, 0.0, 1),
    # row blocks over all columns (configuration 5): three passes over a partial last row
    # block with offsets; two passes with beta and a split K; four passes with long K
    (300, 300, 9000, 3, 8, 0, 1.0, 0.0, 5),
    (257, 130, 20000, 0, 0, 1, 0.5, 1.5, 5),
    (64, 512, 150000, 0, 0, 0, 1.0, 0.0, 5),
]


def _batch(rb, layout, seed=0):
    import torch
    from randblas_gb300 import batched
    g = torch.Generator(device="cuda").manual_seed(seed)
    probs = []
    state = rb.RNGState(7)
    for (d, n, m, ro, co, fam, alpha, beta, cfg) in SHAPES:
        D = rb.DenseDist(d + ro + 3, m + co + 1, rb.ScalarDist(fam))
        S = rb.DenseSkOp(D, state)
        state = S.next_state
        row = layout == rb.Layout.RowMajor
        A = torch.randn(m, n, device="cuda", generator=g)
        B0 = torch.randn(d, n, device="cuda", generator=g)
        if not row:  # column-major storage: keep the matrix, store its transpose's memory
            A = A.t().contiguous()
            B0 = B0.t().contiguous()
        probs.append(batched.BatchProblem(S, A, B0.clone(), d, n, m, alpha, beta, ro, co,
                                          tile_config=cfg))
    return probs


def _plain(rb, p, layout, B0):
    """The same problem through the single-problem plain path."""
    out = B0.clone()
    row = layout == rb.Layout.RowMajor
    lda = p.n if row else p.m
    ldb = p.n if row else p.d
    rb.sketch_general(layout, rb.Op.NoTrans, rb.Op.NoTrans, p.d, p.n, p.m, p.alpha, p.S, p.ro_s,
                      p.co_s, p.A, lda, p.beta, out, ldb)
    return out


@pytest.mark.parametrize("layout", [1, 0])
def test_mixed_batch_matches_plain(rb, oracle, layout):
    import torch
    from oracle.oracle import State
    from randblas_gb300 import batched
    layout = rb.Layout(layout)
    probs = _batch(rb, layout)
    B0 = [p.B.clone() for p in probs]
    refs = [_plain(rb, p, layout, b0) for p, b0 in zip(probs, B0)]
    batched.sketch_batched(probs, layout)
    torch.cuda.synchronize()
    for k, (p, ref) in enumerate(zip(probs, refs)):
        got, want = p.B.double(), ref.double()
        den = max(float(want.norm()), 1e-30)
        rel = float((got - want).norm()) / den
        assert rel < 2e-6, (k, rel)
    # anchor two problems on the oracle (FP64 operator from the reference's algorithm)
    for k in (1, 4):
        p = probs[k]
        d, n, m = p.d, p.n, p.m
        st = p.S.seed_state
        Sfull = oracle.dense_matrix(0, p.S.dist.n_rows, p.S.dist.n_cols, int(p.S.dist.family),
                                    1, State.make(tuple(st.counter), tuple(st.key)))
        Ssub = Sfull[p.ro_s:p.ro_s + d, p.co_s:p.co_s + m].astype(np.float64)
        A = to_host(p.A).astype(np.float64)
        A = A if layout == rb.Layout.RowMajor else A.T
        want = p.alpha * (Ssub @ A)
        b0 = to_host(B0[k]).astype(np.float64)
        b0 = b0 if layout == rb.Layout.RowMajor else b0.T
        want = want + p.beta * b0
        got = to_host(p.B).astype(np.float64)
        got = got if layout == rb.Layout.RowMajor else got.T
        rel = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert rel < 2e-6, (k, rel)


def test_reproducible_plan_and_graph(rb):
    import torch
    from randblas_gb300 import batched
    layout = rb.Layout.RowMajor
    probs = _batch(rb, layout, seed=3)
    for p in probs:
        p.beta = 0.0
    batched.sketch_batched(probs, layout)
    first = [p.B.clone() for p in probs]
    for p in probs:
        p.B.fill_(float("nan"))
    plan = batched.BatchedPlan(probs, layout)
    assert plan.info()["work_items"] >= len(probs)
    plan.execute()
    torch.cuda.synchronize()
    for a, p in zip(first, probs):
        assert torch.equal(a, p.B)
    for p in probs:
        p.B.zero_()
    graph = plan.capture()
    for p in probs:
        p.B.fill_(float("nan"))
    graph.replay()
    graph.replay()
    torch.cuda.synchronize()
    for a, p in zip(first, probs):
        assert torch.equal(a, p.B)
    plan.close()


def test_benchmark_distribution_sampled(rb):
    import torch
    from randblas_gb300 import batched
    rng = np.random.default_rng(0)
    count = 512
    ms = np.round(2.0 ** rng.uniform(12, 18, count)).astype(int)
    ns = rng.integers(16, 513, count)
    g = torch.Generator(device="cuda").manual_seed(0)
    probs, state = [], rb.RNGState(4)
    for i in range(count):
        d, n, m = 4 * int(ns[i]), int(ns[i]), int(ms[i])
        S = rb.DenseSkOp(rb.DenseDist(d, m), state)
        state = S.next_state
        A = torch.randn(m, n, device="cuda", generator=g)
        probs.append(batched.BatchProblem(S, A, torch.empty(d, n, device="cuda"), d, n, m))
    batched.sketch_batched(probs)
    torch.cuda.synchronize()
    for k in rng.choice(count, 8, replace=False):
        p = probs[int(k)]
        want = _plain(rb, p, rb.Layout.RowMajor, torch.zeros_like(p.B)).double()
        rel = float((p.B.double() - want).norm() / want.norm())
        # FP32 sums over up to 2^18 terms, split differently by the two paths
        assert rel < 2e-5, (int(k), rel)


def test_tune_batch_plan_matches_plain(rb, tmp_path):
    """Autotuner.tune_batch on a small mixed batch (beta = 0, so repeated runs give the same
    output): the plan it returns (per-class choices or the library's, whichever ran faster)
    computes every problem to FP32 accuracy, and its problems keep the configurations it uses
    (0 or a valid configuration)."""
    import torch
    from randblas_gb300 import batched
    layout = rb.Layout.RowMajor
    probs = _batch(rb, layout, seed=5)
    for p in probs:
        p.beta = 0.0
        p.tile_config = 0
    refs = [_plain(rb, p, layout, p.B.clone()) for p in probs]
    tuner = batched.Autotuner(cache_path=str(tmp_path / "tiles.json"))
    plan = tuner.tune_batch(probs, layout)
    for p in probs:
        p.B.fill_(float("nan"))
    plan.execute()
    torch.cuda.synchronize()
    plan.close()
    n_cfg = len(batched.tile_configs())
    for k, (p, ref) in enumerate(zip(probs, refs)):
        assert 0 <= p.tile_config <= n_cfg, (k, p.tile_config)
        rel = float((p.B.double() - ref.double()).norm()) / max(float(ref.double().norm()),
                                                                 1e-30)
        assert rel < 2e-6, (k, rel)
