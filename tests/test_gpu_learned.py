"""The learned alpha guess: GPU training kernels against the CPU oracle, the
fused BF16 tensor-core inference against its restatement, and what the guess
changes in the entropic step."""
import numpy as np
import pytest

from oracle import mlp as mlp_oracle


def synthetic(n_in=27, n=3000, seed=0):
    rng = np.random.default_rng(seed)
    X = (rng.standard_normal((n, n_in)) * 1e-3).astype(np.float32)
    y = (2.0 + 0.05 * np.tanh(X[:, :5].sum(1) * 300.0)).astype(np.float32)
    return X, y


def model_for(X, y, seed=1):
    from metalbm_gb300 import MlpModel
    std = X.std(0)
    return MlpModel.init(X.shape[1], (1.0 / std).astype(np.float32), float(np.std(y - 2)), seed)


@pytest.fixture(scope="module")
def lat():
    from metalbm_gb300 import InputDeck, Lattice, build
    build.build()
    with Lattice(InputDeck(latticeT="D3Q27", globalLength=(4, 4, 4))) as L:
        yield L


@pytest.mark.gpu
@pytest.mark.parametrize("n_in", [9, 19, 27])
def test_gradient_matches_cpu_oracle(lat, n_in):
    X, y = synthetic(n_in, 2000)
    m = model_for(X, y)
    loss, g = lat.alpha_model_gradient(m, X, y)
    ref_loss, ref = mlp_oracle.loss_and_grad(m, X, y)
    assert abs(loss - ref_loss) <= 1e-5 * ref_loss
    for k in ("w1", "b1", "w2", "b2", "w3"):
        a, b = getattr(g, k), ref[k]
        assert np.abs(a - b).max() <= 2e-4 * np.abs(b).max() + 1e-9, k
    assert abs(g.b3 - ref["b3"]) <= 2e-4 * abs(ref["b3"]) + 1e-9


@pytest.mark.gpu
def test_gradient_matches_finite_differences(lat):
    X, y = synthetic(27, 500, seed=3)
    m = model_for(X, y, seed=4)
    _, g = lat.alpha_model_gradient(m, X, y)
    rng = np.random.default_rng(0)
    for name in ("w1", "w2", "w3", "b1"):
        arr = getattr(m, name)
        for _ in range(4):
            idx = tuple(rng.integers(0, s) for s in arr.shape)
            h = 1e-3 * max(1.0, abs(float(arr[idx])))
            old = float(arr[idx])
            arr[idx] = old + h
            lp = mlp_oracle.loss_only(m, X, y.astype(np.float64))
            arr[idx] = old - h
            lm = mlp_oracle.loss_only(m, X, y.astype(np.float64))
            arr[idx] = old
            fd = (lp - lm) / (2 * h)
            assert abs(getattr(g, name)[idx] - fd) <= 1e-3 * abs(fd) + 1e-7


@pytest.mark.gpu
@pytest.mark.parametrize("n_in", [9, 19, 27])
def test_tensor_core_inference_matches_bf16_restatement(lat, n_in):
    X, y = synthetic(n_in, 1000, seed=5)
    m = model_for(X, y, seed=6)
    got = lat.alpha_model_predict(m, X)
    ref = mlp_oracle.predict_bf16(m, X)
    err = np.abs(got - ref) / m.output_scale
    # The kernel's tanh is the hardware approximation (absolute error below
    # 2^-10) and its FP32 accumulation order differs, which can move a hidden
    # activation across a bfloat16 rounding boundary (2^-8 relative): the
    # output stays within a few 1e-3 of the BF16 restatement (relative to
    # output_scale), where a layout or indexing error gives O(1).
    assert np.quantile(err, 0.5) <= 1e-3
    assert np.quantile(err, 0.99) <= 5e-3
    assert err.max() <= 2e-2


@pytest.mark.gpu
def test_training_reduces_loss(lat):
    X, y = synthetic(27, 20000, seed=7)
    m0 = model_for(X, y, seed=8)
    l0 = mlp_oracle.loss_only(m0, X, y.astype(np.float64))
    m1, last = lat.train_alpha_model(X, y, m0, epochs=20, batch=2048, lr=3e-3)
    l1 = mlp_oracle.loss_only(m1, X, y.astype(np.float64))
    assert l1 < 0.2 * l0, (l0, l1, last)


def _entropic_run(guess, model=None, steps=6, shape=(16, 12, 10)):
    from metalbm_gb300 import InputDeck, Lattice, fields
    rho, u = fields.taylor_green(shape, u0=0.08)
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.50025,
                     globalLength=shape, storage="f32", alphaSolver="residual",
                     alphaGuess=guess, newtonTolerance=1e-12, deviationThreshold=0.0)
    with Lattice(deck) as L:
        if model is not None:
            L.set_alpha_model(model)
        L.init_equilibrium(rho, u)
        L.step(steps, store=True)
        return L.fields(), L.diagnostics()


@pytest.mark.gpu
def test_zero_model_equals_constant_two_guess():
    """A model with zero weights outputs exactly 2. Run at every node
    (learned_everywhere) it reproduces the constant-2 guess bit for bit; as the
    gated guess (learned: the model only where no solved alpha is stored, i.e.
    after initialisation) it reproduces the previous-alpha guess, whose first
    step starts from the initial alpha = 2."""
    from metalbm_gb300 import MlpModel
    z = MlpModel.init(27, np.ones(27, np.float32), 0.05, seed=0)
    z.w1[:] = 0; z.w2[:] = 0; z.w3[:] = 0; z.b3 = 0.0
    a, da = _entropic_run("learned_everywhere", z)
    b, db = _entropic_run("two")
    assert np.array_equal(a["alpha"], b["alpha"]) and np.array_equal(a["u"], b["u"])
    assert da["newton_iterations"] == db["newton_iterations"]
    assert da["learned_nodes"] == da["solved_nodes"] > 0
    c, dc = _entropic_run("learned", z)
    e, de = _entropic_run("previous")
    assert np.array_equal(c["alpha"], e["alpha"]) and np.array_equal(c["u"], e["u"])
    assert dc["newton_iterations"] == de["newton_iterations"]
    # the network ran on the first step only (the later steps start from a
    # solved alpha)
    assert 0 < dc["learned_nodes"] < dc["solved_nodes"]


@pytest.mark.gpu
def test_learned_kernel_only_where_a_node_lacks_a_solved_alpha():
    """MLBM_GUESS_LEARNED with a zero-weight model (its guess is exactly 2):
    the first call after initialisation runs the network (learned_nodes > 0)
    and matches the previous-alpha guess bit for bit; a later call starts with
    every alpha solved and runs the kernels without the network
    (learned_nodes = 0), still bit for bit; after mlbm_set_alpha with nodes
    at alpha = 2 the next call runs the network on those (the solved ones of
    them)."""
    from metalbm_gb300 import InputDeck, Lattice, MlpModel, fields
    z = MlpModel.init(27, np.ones(27, np.float32), 0.05, seed=0)
    z.w1[:] = 0; z.w2[:] = 0; z.w3[:] = 0; z.b3 = 0.0
    shape = (16, 12, 10)
    rho, u = fields.taylor_green(shape, u0=0.08)
    out = {}
    for guess in ("learned", "previous"):
        deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.50025,
                         globalLength=shape, storage="f32", alphaSolver="residual",
                         alphaGuess=guess, newtonTolerance=1e-12, deviationThreshold=0.0)
        with Lattice(deck) as L:
            if guess == "learned":
                L.set_alpha_model(z)
            L.init_equilibrium(rho, u)
            L.step(2)
            d1 = L.diagnostics()
            L.step(3, store=True)
            d2 = L.diagnostics()
            f2 = L.fields()
            a = f2["alpha"].copy()
            a[:100] = 2.0  # 100 nodes without a solved alpha
            L.set_alpha(a)
            L.step(1)
            d3 = L.diagnostics()
            out[guess] = (d1, d2, f2, d3, L.populations())
    dl, dp = out["learned"], out["previous"]
    assert dl[0]["learned_nodes"] > 0 and dp[0]["learned_nodes"] == 0
    assert dl[1]["learned_nodes"] == 0
    assert dl[1]["newton_iterations"] == dp[1]["newton_iterations"]
    assert np.array_equal(dl[2]["alpha"], dp[2]["alpha"]) and np.array_equal(dl[2]["u"], dp[2]["u"])
    assert 0 < dl[3]["learned_nodes"] <= 100 and dp[3]["learned_nodes"] == 0
    assert np.array_equal(dl[4], dp[4])


@pytest.mark.gpu
def test_learned_guess_at_equal_residual():
    """Train on samples of a plain run (the library's sample logger and GPU
    training kernels), then start from the initial state, where no node has a
    solved alpha: the network's guesses start the solve closer to the roots
    than the constant 2 the reference starts from (Initialize.h:82-89): they
    pass the residual test |F| <= 1e-12 at least as often and save Newton
    iterations; and the steps that
    follow (the previous alpha wherever one is solved) agree with the plain
    run to 1e-6 in u without the alpha = 2 fallback."""
    from metalbm_gb300 import InputDeck, fields
    from metalbm_gb300 import alpha_model
    shape = (16, 12, 10)
    rho, u = fields.taylor_green(shape, u0=0.08)
    deck = InputDeck(latticeT="D3Q27", collisionT="ELBM", relaxationTime=0.50025,
                     globalLength=shape, storage="f32", alphaSolver="residual",
                     alphaGuess="two", newtonTolerance=1e-12, deviationThreshold=0.0)
    # every step logged, the first one (the state the cold start sees) included
    X, y = alpha_model.collect_samples(deck, rho, u, steps=12, every=1, n_per_log=1920)
    model, loss = alpha_model.fit(X, y, deck, epochs=120, batch=1024, lr=3e-3)
    assert np.sqrt(loss) < np.std(y)  # the model explains part of alpha*
    # the first step from the initial state: network against alpha = 2
    _, d1 = _entropic_run("learned", model, steps=1)
    _, d2 = _entropic_run("two", steps=1)
    assert d1["learned_nodes"] == d1["solved_nodes"] == d2["solved_nodes"] > 0
    assert d1["guess_hits"] >= d2["guess_hits"]
    assert d1["newton_iterations"] < d2["newton_iterations"]
    # a run of steps at the same residual
    a, da = _entropic_run("learned", model)
    b, db = _entropic_run("two")
    assert da["fallback_nodes"] == 0 and db["fallback_nodes"] == 0
    assert da["solved_nodes"] == db["solved_nodes"] > 0
    assert np.abs(a["u"] - b["u"]).max() <= 1e-6
    print("first step: newton iterations learned/two:", d1["newton_iterations"],
          d2["newton_iterations"], "guess hits learned/two:", d1["guess_hits"], d2["guess_hits"])
