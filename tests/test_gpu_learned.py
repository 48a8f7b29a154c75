"""The learned 4x-dt stepper on the GPU (include/clsph_learned.h).

* the BF16 tensor-core MLP against a plain PyTorch fp32 reference of the same
  network (forward, and the gradients of one training pass);
* training reduces the loss of a smooth synthetic regression;
* the neighbour features against a numpy restatement;
* the learned step with a zero network is the plain solver at 4x dt, bit for
  bit (oracle run with simulation_scale x 4); with a zero threshold every
  learned step is rolled back and the result is the plain trajectory;
* the sample collector leaves the trajectory unchanged and its targets obey
  their definitions.
"""

import numpy as np
import pytest

from libclsph_gb300 import learned as Lm
from libclsph_gb300 import workloads as W
from libclsph_gb300.gpu import STAGE_FORCES, GpuSolver

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def random_blob(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    b = np.zeros(Lm.BLOB, dtype=np.float32)
    b[Lm.OFF_W1:Lm.OFF_B1] = rng.normal(0, np.sqrt(2 / 32), 32 * 256) * scale
    b[Lm.OFF_B1:Lm.OFF_W2] = rng.normal(0, 0.1, 256)
    b[Lm.OFF_W2:Lm.OFF_B2] = rng.normal(0, np.sqrt(2 / 256), 256 * 256) * scale
    b[Lm.OFF_B2:Lm.OFF_W3] = rng.normal(0, 0.1, 256)
    b[Lm.OFF_W3:Lm.OFF_B3] = rng.normal(0, np.sqrt(1 / 256), 256 * 4)
    b[Lm.OFF_B3:Lm.N_PARAMS] = rng.normal(0, 0.1, 4)
    b[Lm.OFF_XMU:Lm.OFF_XSIGMA] = rng.normal(0, 0.5, 32)
    b[Lm.OFF_XSIGMA:Lm.OFF_YMU] = rng.uniform(0.5, 2.0, 32)
    b[Lm.OFF_YMU:Lm.OFF_YSIGMA] = rng.normal(0, 0.5, 4)
    b[Lm.OFF_YSIGMA:Lm.BLOB] = rng.uniform(0.5, 2.0, 4)
    return b


def gelu_bf16(z):
    """The kernels' GELU: inputs, constants and every intermediate in BF16
    (tanh form), result BF16 (returned as fp32 values)."""
    bf = torch.bfloat16
    k0 = torch.tensor(0.7978845608028654, dtype=torch.float32).to(bf).float()
    k01 = torch.tensor(0.7978845608028654 * 0.044715, dtype=torch.float32).to(bf).float()
    x = z.detach().to(bf).float()
    x2 = (x * x).to(bf).float()
    c = (x2 * k01 + k0).to(bf).float()
    u = (x * c).to(bf).float()
    t = torch.tanh(u).to(bf).float()
    hx = (x * 0.5).to(bf).float()
    return (hx * t + hx).to(bf).float()


def torch_mlp(blob, ste=False):
    """fp32 PyTorch reference of the network with the kernels' BF16 roundings
    (weights, input rows, both hidden activations)."""
    t = torch.tensor(blob, dtype=torch.float32, device="cuda")
    parts = {
        "w1": t[Lm.OFF_W1:Lm.OFF_B1].view(32, 256), "b1": t[Lm.OFF_B1:Lm.OFF_W2],
        "w2": t[Lm.OFF_W2:Lm.OFF_B2].view(256, 256), "b2": t[Lm.OFF_B2:Lm.OFF_W3],
        "w3": t[Lm.OFF_W3:Lm.OFF_B3].view(256, 4), "b3": t[Lm.OFF_B3:Lm.N_PARAMS],
    }
    if ste:
        for k in parts:
            parts[k] = parts[k].clone().requires_grad_(True)

    def q(x):  # bf16 rounding with a straight-through gradient
        return x + (x.to(torch.bfloat16).float() - x).detach()

    def act(z):  # the kernels' packed-BF16 GELU forward, the tanh-GELU derivative backward
        g = torch.nn.functional.gelu(z, approximate="tanh")
        return g + (gelu_bf16(z) - g).detach()

    def fwd(x_std):
        h1 = act(x_std @ q(parts["w1"]) + parts["b1"])
        h2 = act(h1 @ q(parts["w2"]) + parts["b2"])
        return h2 @ q(parts["w3"]) + parts["b3"]

    return fwd, parts, t


def test_forward_matches_torch(gpu_lib):
    blob = random_blob(1)
    rows = 5000  # not a multiple of 16: exercises the ragged last tile
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(rows, 32, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    y = torch.empty(rows, 4, device="cuda", dtype=torch.float32)
    m = Lm.Mlp(blob=blob)
    m.forward(x.data_ptr(), rows, y.data_ptr())
    y_mma = torch.empty_like(y)
    m.forward_mma_sync(x.data_ptr(), rows, y_mma.data_ptr())
    torch.cuda.synchronize()
    assert m.status() == 0
    with torch.no_grad():
        fwd, _, t = torch_mlp(blob)
        ref = fwd(x.float()) * t[Lm.OFF_YSIGMA:] + t[Lm.OFF_YMU:Lm.OFF_YSIGMA]
    scale = ref.abs().max().item()
    for got, want in ((y, ref), (y_mma, ref)):
        err = (got - want).abs()
        assert err.max().item() <= 1e-2 * scale, (err.max().item(), scale)
        assert err.mean().item() <= 1e-3 * scale, (err.mean().item(), scale)
    m.close()


@pytest.mark.parametrize("tiles_per_cta", [2, 3, 7])
def test_forward_many_tiles_per_cta(gpu_lib, tiles_per_cta):
    """Enough rows for several 128-row tiles per persistent CTA, so the
    tcgen05 kernel's two tensor-memory regions alternate and its two-tile
    pipeline runs in steady state, with a ragged last tile; it must agree
    with the mma.sync kernel and with the PyTorch restatement."""
    blob = random_blob(3 + tiles_per_cta)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    rows = sms * 128 * tiles_per_cta - 51
    g = torch.Generator(device="cuda").manual_seed(tiles_per_cta)
    x = torch.randn(rows, 32, device="cuda", generator=g).to(torch.bfloat16).contiguous()
    y = torch.empty(rows, 4, device="cuda", dtype=torch.float32)
    y_mma = torch.empty_like(y)
    m = Lm.Mlp(blob=blob)
    m.forward(x.data_ptr(), rows, y.data_ptr())
    m.forward_mma_sync(x.data_ptr(), rows, y_mma.data_ptr())
    torch.cuda.synchronize()
    assert m.status() == 0
    with torch.no_grad():
        fwd, _, t = torch_mlp(blob)
        ref = fwd(x.float()) * t[Lm.OFF_YSIGMA:] + t[Lm.OFF_YMU:Lm.OFF_YSIGMA]
    scale = ref.abs().max().item()
    for got in (y, y_mma):
        err = (got - ref).abs()
        assert err.max().item() <= 1e-2 * scale, (err.max().item(), scale)
        assert err.mean().item() <= 1e-3 * scale, (err.mean().item(), scale)
    # the two tensor-core paths round the same BF16 products: close to each other
    assert (y - y_mma).abs().max().item() <= 1e-2 * scale
    m.close()


def test_gradients_match_torch(gpu_lib):
    blob = random_blob(2)
    rows = 4096
    g = torch.Generator(device="cuda").manual_seed(1)
    x_raw = torch.randn(rows, 32, device="cuda", generator=g) * 1.5 + 0.3
    y_raw = torch.randn(rows, 4, device="cuda", generator=g)
    m = Lm.Mlp(blob=blob)
    grads, loss = m.gradients(x_raw.data_ptr(), y_raw.data_ptr(), rows)
    fwd, parts, t = torch_mlp(blob, ste=True)
    x_std = ((x_raw - t[Lm.OFF_XMU:Lm.OFF_XSIGMA]) / t[Lm.OFF_XSIGMA:Lm.OFF_YMU]).clamp(-6, 6)
    x_std = x_std.to(torch.bfloat16).float()
    y_std = (y_raw - t[Lm.OFF_YMU:Lm.OFF_YSIGMA]) / t[Lm.OFF_YSIGMA:]
    ref_loss = ((fwd(x_std) - y_std) ** 2).sum(1).mean()
    ref_loss.backward()
    assert abs(loss - ref_loss.item()) <= 3e-3 * ref_loss.item()
    offs = {"w1": (Lm.OFF_W1, Lm.OFF_B1), "b1": (Lm.OFF_B1, Lm.OFF_W2), "w2": (Lm.OFF_W2, Lm.OFF_B2),
            "b2": (Lm.OFF_B2, Lm.OFF_W3), "w3": (Lm.OFF_W3, Lm.OFF_B3), "b3": (Lm.OFF_B3, Lm.N_PARAMS)}
    for k, (a, b) in offs.items():
        ref = parts[k].grad.detach().reshape(-1).cpu().numpy().astype(np.float64)
        got = grads[a:b].astype(np.float64)
        rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
        assert rel <= 3e-2, (k, rel)
    m.close()


def test_training_reduces_loss(gpu_lib):
    rows = 1 << 17
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(rows, 32, device="cuda", generator=g)
    w = torch.randn(32, 4, device="cuda", generator=g) / 4
    y = torch.tanh(x @ w)
    m = Lm.Mlp(seed=5)
    log = m.train(x.data_ptr(), y.data_ptr(), rows, epochs=40, batch=8192, lr=2e-3, lr_final=1e-4,
                  log_every=32)
    after = m.loss(x.data_ptr(), y.data_ptr(), rows)  # with the fitted normalisation
    assert np.isfinite(log).all() and len(log) > 4
    assert log[-1] < 0.1 * log[0], log
    # standardised targets have unit variance per output, so predicting the mean scores 4
    assert after < 0.1, after
    m.close()


def features_numpy(pos, vel, ivel, rho, prs, acc, params):
    """Restatement of the 32 features in float64 from the sorted state; the
    neighbour set is the density kernel's: float32 r = sqrt((dx^2 + dy^2) + dz^2) < h;
    pair moments from the velocity, own-velocity features from the
    intermediate velocity."""
    h = np.float32(params["h"])
    dt = float(np.float32(params["time_delta"]) * np.float32(params["simulation_scale"]))
    rho0, K, vmax = float(params["fluid_density"]), float(params["K"]), float(params["max_velocity"])
    n = len(pos)
    out = np.zeros((n, 32))
    vs = dt / float(h)
    for i in range(n):
        d32 = (pos[i] - pos).astype(np.float32)
        r = np.sqrt((d32[:, 0] * d32[:, 0] + d32[:, 1] * d32[:, 1]) + d32[:, 2] * d32[:, 2])
        nb = np.nonzero(r < h)[0]
        cnt = len(nb)
        nb = nb[nb != i]
        d = (pos[nb].astype(np.float64) - pos[i]) / float(h)
        u = (vel[nb].astype(np.float64) - vel[i]) * vs
        w = np.maximum(0.0, 1.0 - (d ** 2).sum(1))
        f = out[i]
        f[0] = rho[i] / rho0 - 1
        f[1] = prs[i] / K
        f[2] = cnt / 32
        f[3:6] = acc[i] * dt * dt / float(h)
        f[6:9] = ivel[i] * vs
        f[9] = np.linalg.norm(ivel[i].astype(np.float64)) / vmax
        f[10:13] = (w[:, None] * d).sum(0)
        f[13:19] = [(w * d[:, 0] ** 2).sum(), (w * d[:, 1] ** 2).sum(), (w * d[:, 2] ** 2).sum(),
                    (w * d[:, 0] * d[:, 1]).sum(), (w * d[:, 0] * d[:, 2]).sum(), (w * d[:, 1] * d[:, 2]).sum()]
        f[19:22] = (w[:, None] * u).sum(0)
        f[22:28] = [(w * u[:, 0] ** 2).sum(), (w * u[:, 1] ** 2).sum(), (w * u[:, 2] ** 2).sum(),
                    (w * u[:, 0] * u[:, 1]).sum(), (w * u[:, 0] * u[:, 2]).sum(), (w * u[:, 1] * u[:, 2]).sum()]
        f[28] = (w * (d * u).sum(1)).sum()
        f[29:32] = (w[:, None] * np.cross(d, u)).sum(0)
    return out


def test_features_match_numpy(gpu_lib):
    sc = W.small_block(10, seed=5, velocity_sigma=0.3)
    parts = sc.particles.copy()  # velocity and intermediate velocity differ
    parts["velocity"][:, :3] += np.random.default_rng(9).normal(0, 0.2, (sc.n, 3)).astype(np.float32)
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(parts)
        g.step_until(STAGE_FORCES)
        _, perm = g.keys()
        rho, prs, acc = g.fields()
        feats = Lm.read_features(g)
    pos = parts["position"][perm, :3]
    vel = parts["velocity"][perm, :3]
    ivel = parts["intermediate_velocity"][perm, :3]
    ref = features_numpy(pos, vel, ivel, rho, prs, acc[:, :3], sc.params)
    scale = np.abs(ref).max(0) + 1e-12
    err = (np.abs(feats - ref) / scale).max(0)
    assert (err <= 1e-4).all(), {Lm.FEATURE_NAMES[k]: float(err[k]) for k in np.nonzero(err > 1e-4)[0]}


def identity_blob():
    b = np.zeros(Lm.BLOB, dtype=np.float32)
    b[Lm.OFF_XSIGMA:Lm.OFF_YMU] = 1
    b[Lm.OFF_YSIGMA:Lm.BLOB] = 1
    return b


def scene_for_steps():
    return W.small_block(12, seed=4, velocity_sigma=0.3, offset=(0.2, 0.01, 0.2))


def test_zero_network_single_dt_is_plain_solver(gpu_lib, oracle):
    """dt_mult = 1, zero network: the learned step is the plain substep, bit for bit."""
    sc = scene_for_steps()
    m = Lm.Mlp(blob=identity_blob())
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        st = Lm.step_learned(g, m, 3, dt_mult=1, threshold=1e30)
        out = g.download()
    assert st.learned_steps == 3 and st.rejected == 0 and st.plain_substeps == 0
    ref = oracle.run(sc.params, sc.terms, sc.particles, 3, sc.mesh)
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], ref[f][:, :3]), f
    m.close()


def test_zero_network_4dt_reproduces_constant_acceleration(gpu_lib):
    """Particles out of each other's reach feel gravity only: one 4-dt step with
    the weighted position update lands where 4 plain substeps do."""
    sc = W.small_block(6, seed=7, velocity_sigma=0.2, offset=(0.2, 0.3, 0.2), spacing_frac=1.6)
    m = Lm.Mlp(blob=identity_blob())
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as a, GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as b:
        a.upload(sc.particles)
        b.upload(sc.particles)
        Lm.step_learned(a, m, 3, dt_mult=4, threshold=1e30)
        b.step(12)
        la, pb = a.download(), b.download()
        ia, ib = a.ids(), b.ids()
    la, pb = la[np.argsort(ia)], pb[np.argsort(ib)]
    for f in ("position", "intermediate_velocity"):
        assert np.allclose(la[f][:, :3], pb[f][:, :3], rtol=1e-5, atol=1e-6), f
    m.close()


def test_zero_threshold_rolls_back_to_plain(gpu_lib, oracle):
    sc = scene_for_steps()
    m = Lm.Mlp(blob=identity_blob())
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as g:
        g.upload(sc.particles)
        st = Lm.step_learned(g, m, 3, dt_mult=4, threshold=0.0)
        out = g.download()
    assert st.rejected == 3 and st.learned_steps == 0 and st.plain_substeps == 12
    ref = oracle.run(sc.params, sc.terms, sc.particles, 12, sc.mesh)
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(out[f][:, :3], ref[f][:, :3]), f
    m.close()


def test_collector_keeps_trajectory_and_targets(gpu_lib):
    sc = W.small_block(16, seed=6, velocity_sigma=0.2, offset=(0.2, 0.2, 0.2))
    stride, steps, mult = 8, 12, 4
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as a, GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as b:
        a.upload(sc.particles)
        b.upload(sc.particles)
        c = Lm.Collector(a, stride, capacity=1 << 20, dt_mult=mult)
        c.step(steps)
        b.step(steps)
        pa, pb = a.download(), b.download()
        x, y = c.copy()
        c.close()
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(pa[f], pb[f]), f
    m = (sc.n + stride - 1) // stride
    assert x.shape == (m * (steps - mult), 32) and y.shape == (m * (steps - mult), 4)
    x = x.reshape(steps - mult, m, 32).astype(np.float64)
    y = y.reshape(steps - mult, m, 4).astype(np.float64)
    # density target: rho(t + 4 dt) / rho(t) - 1, from the features 4 substeps apart
    k = steps - 2 * mult
    dr = (x[mult:mult + k, :, 0] + 1) / (x[:k, :, 0] + 1) - 1
    assert np.allclose(y[:k, :, 3], dr, rtol=1e-5, atol=1e-6)
    # velocity target without clamp or collision: (v(t+4) - v(t)) / 4 - a(t), units h/dt^2
    dv = (x[mult:mult + k, :, 6:9] - x[:k, :, 6:9]) / mult - x[:k, :, 3:6]
    close = np.isclose(y[:k, :, :3], dv, rtol=1e-3, atol=1e-4 * np.abs(dv).max())
    assert close.mean() > 0.9, close.mean()


def test_no_check_run_equals_unlimited_check(gpu_lib):
    """check=False (no snapshots, gates or host waits) advances the state
    exactly as a check that never fires, launched step by step and replayed
    from CUDA graphs of 4 steps (9 steps: two replays and one launched step;
    then 4 more with another network, which rebuilds the graph)."""
    sc = W.small_block(12, seed=9, velocity_sigma=0.3, offset=(0.2, 0.05, 0.2))
    m = Lm.Mlp(blob=random_blob(4, scale=0.05))
    m2 = Lm.Mlp(blob=random_blob(5, scale=0.05))
    solvers = [GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) for _ in range(3)]
    try:
        a, b, c = solvers
        for s in solvers:
            s.upload(sc.particles)
        c.set_graph(True)
        sa = Lm.step_learned(a, m, 9, threshold=1e30)
        sb = Lm.step_learned(b, m, 9, check=False)
        sc_ = Lm.step_learned(c, m, 9, check=False)
        for s in solvers[1:]:
            Lm.step_learned(s, m2, 4, check=False)
        Lm.step_learned(a, m2, 4, threshold=1e30)
        pa, pb, pc = (s.download() for s in solvers)
    finally:
        for s in solvers:
            s.close()
    assert sa.learned_steps == sb.learned_steps == sc_.learned_steps == 9
    assert sb.checks == 0 and sb.rejected == 0
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(pa[f][:, :3], pb[f][:, :3]), f
        assert np.array_equal(pa[f][:, :3], pc[f][:, :3]), f
    m.close()
    m2.close()


def test_collector_on_learned_rollout(gpu_lib):
    """Sampling along learned steps leaves the learned trajectory unchanged and
    yields one sample per tracked particle per learned step."""
    sc = W.small_block(12, seed=8, velocity_sigma=0.2, offset=(0.2, 0.2, 0.2))
    m = Lm.Mlp(blob=random_blob(3, scale=0.05))
    stride, steps = 4, 3
    with GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as a, GpuSolver(sc.params, sc.terms, sc.n, sc.mesh) as b:
        a.upload(sc.particles)
        b.upload(sc.particles)
        c = Lm.Collector(a, stride, capacity=1 << 20)
        c.step_learned(m, steps)
        Lm.step_learned(b, m, steps, threshold=1e30)
        pa, pb = a.download(), b.download()
        count = c.samples()[2]
        x, y = c.copy()
        c.close()
    for f in ("position", "velocity", "intermediate_velocity"):
        assert np.array_equal(pa[f][:, :3], pb[f][:, :3]), f
    assert count == steps * ((sc.n + stride - 1) // stride)
    assert np.isfinite(x).all() and np.isfinite(y).all()
    m.close()


def _committed_runs(sc, substeps=400):
    from libclsph_gb300.stepper_eval import evaluate

    path = Lm.default_weights_path()
    if not path.exists():
        pytest.skip("no committed weights")
    net = Lm.Mlp.load(path)
    zero = Lm.Mlp(blob=identity_blob())  # every output 0: the bare 4 dt step
    try:
        runs = {"checked": evaluate(sc, net, plain_substeps=substeps, checkpoints=4, threshold=0.01),
                "free": evaluate(sc, net, plain_substeps=substeps, checkpoints=4, check=False),
                "zero": evaluate(sc, zero, plain_substeps=substeps, checkpoints=4, check=False)}
    finally:
        net.close()
        zero.close()
    print(sc.name, "(density_dev, max, fallback, pos_rms_h):",
          {k: (r["density_dev"], r["density_dev_max"], r["fallback_fraction"], r["pos_rms_h_final"])
           for k, r in runs.items()})
    for r in runs.values():
        assert np.isfinite(r["density_dev"]) and np.isfinite(r["pos_rms_h_final"])
    return runs


def test_committed_weights_fall_back_outside_their_training_scenes(gpu_lib):
    """The committed network (libclsph_gb300/weights/stepper_4dt.npz) was
    trained on dam breaks with h = 1/64 m; the 32,768-particle dam break has
    h = 0.062 m, outside that distribution, where the network's corrections
    are worse than none (measured on a GB300: 22 % density deviation free
    running against 8 % for the bare 4 dt step). The 1 % density check must
    then roll every learned step back: the checked run stays on the plain
    trajectory."""
    runs = _committed_runs(W.dam_break_32k())
    checked = runs["checked"]
    assert checked["fallback_fraction"] >= 0.9
    assert checked["density_dev"] <= 0.01
    assert checked["pos_rms_h_final"] <= 0.5


def test_committed_weights_on_a_training_like_dam_break(gpu_lib):
    """The committed network on a dam break of its training distribution
    (h = 1/64 m, a 64 x 64 x 32 column in the left quarter of a 2 x 1 x 1 m
    box, 131,072 particles) over 400 plain substeps' time. Measured on a
    GB300 when this test was written: with the 1 % check 99 % of the learned
    steps roll back and the run stays within 0.3 % density deviation of the
    plain solver; free running the network deviates 5.6 %, more than the
    bare 4 dt step's 1.5 % (its single-step corrections do not survive
    rollout). The bounds pin that behaviour: the check keeps the run within
    1 %, and the free run does not get worse than 8 %."""
    sc = W.dam_break((64, 64, 32), box=(2.0, 1.0, 1.0), seed=9)
    runs = _committed_runs(sc)
    assert runs["checked"]["density_dev"] <= 0.01
    assert runs["free"]["density_dev"] <= 0.08
    assert runs["zero"]["density_dev"] <= 0.03
