"""Train the warm-start network on solve pairs captured from the solver, export it, evaluate it.

    python -m waves_gb300.learned.train --seeds 8 --pairs 40 --out model.npz [--eval-seeds 2] [--trainer torch]

The 2000-pair learned configuration (seeds 1..20, 100 pairs each over t in [2, 10] s; held-out
seeds 101..105; one 24^3 crop per pair, cut while capturing):

    python -m waves_gb300.learned.train --seeds 20 --pairs 100 --t0 2 --gap 0.08 --crops 2000 --eval-seeds 5

Capture: for each seed the 310x48x80 beach (the lab settings) runs with a wave amplitude drawn
from U(0.04, 0.10) m and a period from U(1.2, 1.8) s (wavenumber by the same dispersion
bisection as the presets, std::mt19937_64-independent: numpy's PCG64 seeded with the seed).  It
advances in the CUDA-graph path to the sampling times and takes one trial through the
host-driven phases of include/waves_debug.h: after op 2 the candidate F and p_prev, after the CG
set-up b, and at the first round's convergence (relative residual 1e-6) p*.

Training, --trainer cuda (default): the library's own kernels (k_train.cu, waves_net_train) run
full-batch Adam on a fixed set of random crops with the MSE objective below, as implicit GEMMs on
the tensor cores (--arithmetic tensor, default) or in the oracle's FP32/FP64 order (exact).
--trainer torch: PyTorch, offline: the network of k_net.cu (3x3x3 convolutions 3 -> 16 -> 16 -> 16 -> 1,
ReLU, zero padding) maps (F, b * s_b, p_prev * s_p) to (p* - p_prev) / s_out on wet cells, with
s_b, s_p, s_out the inverse standard deviations / standard deviation of the training data.  The
default objective is the initial residual the solver will see, |r0 - A (s_out y)|^2 / |r0|^2 over
wet cells with r0 = b - A p_prev and A the ghost-fluid operator of operator_at (the residual guard
of the solver compares exactly this norm); --objective mse fits (p* - p_prev) / s_out instead.
Both are scored on random 40x32x32 crops away from the crop edge (the receptive field is 4 cells).
Export: BF16 weights [co][kz][ky][kx][ci], FP32 biases, the scales.

Evaluation: held-out seeds run the same number of steps with and without the network; the
result line gives CG iterations and pressure milliseconds per step for both.
"""
import argparse
import json
import math
import os
import time

import numpy as np

import waves_gb300 as wg
from waves_gb300.learned import CHANNELS, bf16_bits, load_model

DEPTH = 0.45
WITH_COEF = True  # capture the ghost-fluid face coefficients (needed by the residual objective)


def beach(seed, warm=0):
    rng = np.random.default_rng(seed)
    amplitude, period = rng.uniform(0.04, 0.10), rng.uniform(1.2, 1.8)
    cfg = wg.config("beach", pressure_tolerance=1e-6, warm_start=warm)
    cfg.wave[0] = amplitude
    cfg.wave[1] = wg.dispersion_k(period, DEPTH)
    cfg.wave[2] = 2.0 * math.pi / period
    cfg.wave[3] = DEPTH
    return cfg, amplitude, period


def capture_trial(s, N, NF, with_coef=WITH_COEF):
    """One trial through the debug phases; the first round's (F, b, p_prev, p*, kind) or None."""
    s.debug_phase(0)
    c = s.control()
    if not c[4] > 0.5:
        return None
    for phase in (1, 2, 2, 2, 3, 4, 5, 6):
        s.debug_phase(phase)
    cand = 1 - int(c[0])
    bank = s.bank(cand)
    F, p_prev = bank[:N].copy(), bank[N + NF:N + NF + N].copy()
    kind = s.geometry()[1].copy()
    coef = s.debug_read("coef", 6 * N) if with_coef else None
    s.debug_phase(7)
    pair, rounds = None, 0
    while True:
        s.debug_phase(8)
        b = s.debug_read("b", N) if rounds == 0 else None
        c = s.control()
        while c[4] > 0.5 and c[6] < 0.5 and c[7] < 0.5:
            s.debug_phase(9)
            c = s.control()
        if rounds == 0 and c[6] > 0.5 and c[7] < 0.5:
            p_star = s.bank(cand)[N + NF:N + NF + N].copy()
            pair = {"F": F, "b": b, "p_prev": p_prev, "p_star": p_star, "kind": kind, "coef": coef}
        s.debug_phase(10)
        c = s.control()
        rounds += 1
        if not (c[57] == 1 and c[7] < 0.5 and c[4] > 0.5):
            break
    s.debug_phase(11)
    return pair


def capture(seeds, pairs, t0, gap, sink=None, with_coef=WITH_COEF):
    """`pairs` solve pairs per seed at t0 + gap, t0 + 2 gap, ...: the list of pairs, or, with a
    sink, each pair handed to sink(pair) as it is captured (none kept) and the count returned."""
    out, count = [], 0
    for seed in seeds:
        cfg, a, T = beach(seed)
        s = wg.WavesSolver(cfg)
        N, NF = s.N, s.NF
        s.request_time(t0)
        s.run()
        for k in range(pairs):
            s.request_time(t0 + (k + 1) * gap)
            s.run()
            s.request_steps(int(s.control()[2]) + 1)
            p = capture_trial(s, N, NF, with_coef)
            if p is not None:
                count += 1
                if sink is None:
                    out.append(p)
                else:
                    sink(p)
        s.close()
        print(f"seed {seed}: a {a:.3f} m, T {T:.3f} s, {count} pairs so far", flush=True)
    return out if sink is None else count


class CropBank:
    """Training crops cut from solve pairs as they are captured, so that no full pair is kept
    (a beach pair is 24 MB; 2000 of them would not fit in host memory).  Each pair gives
    `rate` crops on average (floor(rate), plus one with probability frac(rate)) at uniform random
    offsets: F, b, p_prev and p* - p_prev, and the loss mask (wet cells at least `edge` cells inside
    the crop).  The input and output scales are the population standard deviations over every wet
    cell of every pair, from running sums."""

    def __init__(self, n, rate, crop=(24, 24, 24), edge=4, seed=0):
        self.nx, self.ny, self.nz = n
        self.cx, self.cy, self.cz = min(crop[0], self.nx), min(crop[1], self.ny), min(crop[2], self.nz)
        self.rate = float(rate)
        self.rng = np.random.default_rng(seed)
        self.inner = np.zeros((self.cz, self.cy, self.cx), np.float32)
        self.inner[edge:self.cz - edge, edge:self.cy - edge, edge:self.cx - edge] = 1.0
        self.raw = []
        self.sums = np.zeros((3, 3))  # rows b, p_prev, p* - p_prev: count, sum, sum of squares
        self.pairs = 0

    def add(self, p):
        grid = lambda a: np.asarray(a, dtype=np.float32).reshape(self.nz, self.ny, self.nx)
        wet = grid(p["kind"]) > 0
        F, b, pp = grid(p["F"]), grid(p["b"]), grid(p["p_prev"])
        dp = grid(p["p_star"]) - pp
        for row, a in enumerate((b, pp, dp)):
            v = a[wet].astype(np.float64)
            self.sums[row] += (v.size, v.sum(), float(np.dot(v, v)))
        whole = int(self.rate)
        count = whole + (1 if self.rng.random() < self.rate - whole else 0)
        for _ in range(count):
            ox = int(self.rng.integers(self.nx - self.cx + 1))
            oy = int(self.rng.integers(self.ny - self.cy + 1))
            oz = int(self.rng.integers(self.nz - self.cz + 1))
            sl = (slice(oz, oz + self.cz), slice(oy, oy + self.cy), slice(ox, ox + self.cx))
            self.raw.append((F[sl].copy(), b[sl].copy(), pp[sl].copy(), dp[sl].copy(),
                             (wet[sl] * self.inner).astype(np.float32)))
        self.pairs += 1

    def scales(self):
        """(s_b, s_p, s_out): inputs are multiplied by s_b and s_p, the target divided by s_out."""
        def std(row):
            n, s1, s2 = self.sums[row]
            return math.sqrt(max(s2 / max(n, 1.0) - (s1 / max(n, 1.0)) ** 2, 0.0))
        return 1.0 / max(std(0), 1e-12), 1.0 / max(std(1), 1e-12), max(std(2), 1e-12)

    def batch(self):
        """(x [crops][3][z][y][x], target, mask, scales) with the scales applied."""
        s_b, s_p, s_out = self.scales()
        k = len(self.raw)
        xs = np.zeros((k, 3, self.cz, self.cy, self.cx), np.float32)
        ys = np.zeros((k, self.cz, self.cy, self.cx), np.float32)
        ms = np.zeros((k, self.cz, self.cy, self.cx), np.float32)
        for i, (F, b, pp, dp, m) in enumerate(self.raw):
            xs[i, 0] = F
            xs[i, 1] = b * s_b
            xs[i, 2] = pp * s_p
            ys[i] = dp / s_out
            ms[i] = m
        return xs, ys, ms, (s_b, s_p, s_out)


def build_net(torch):
    layers = []
    for l, (ci, co) in enumerate(CHANNELS):
        layers.append(torch.nn.Conv3d(ci, co, 3, padding=1))
        if l < len(CHANNELS) - 1:
            layers.append(torch.nn.ReLU())
    return torch.nn.Sequential(*layers)


def apply_operator(torch, x, coef, wet, periodic_x=False):
    """operator_at (pressure_core.glslinc:98-104) on [B, 1, z, y, x] fields: sum over the six faces
    of coef_f * (x_here - x_neighbour), neighbours outside or dry contributing zero, z periodic."""
    xw = x * wet
    out = torch.zeros_like(x)
    for f, (dim, sign) in enumerate(((4, -1), (4, 1), (3, -1), (3, 1), (2, -1), (2, 1))):
        if dim == 2 or (dim == 4 and periodic_x):
            other = torch.roll(xw, shifts=-sign, dims=dim)
        else:
            pad = [0, 0, 0, 0, 0, 0]
            k = 2 * (4 - dim) + (1 if sign > 0 else 0)  # pad the far side of the shifted axis
            pad[k] = 1
            other = torch.nn.functional.pad(xw, pad)
            idx = [slice(None)] * 5
            idx[dim] = slice(1, None) if sign > 0 else slice(0, -1)
            other = other[tuple(idx)]
        out = out + coef[:, f:f + 1] * (xw - other)
    return out * wet


def train(pairs, n, steps, seed, device, objective="residual"):
    import torch
    torch.manual_seed(seed)
    nx, ny, nz = n
    grid = lambda a: torch.from_numpy(a.reshape(nz, ny, nx)).to(device)
    wet = torch.stack([grid(p["kind"]) > 0 for p in pairs])
    b = torch.stack([grid(p["b"]) for p in pairs])
    pp = torch.stack([grid(p["p_prev"]) for p in pairs])
    dp = torch.stack([grid(p["p_star"]) for p in pairs]) - pp
    F = torch.stack([grid(p["F"]) for p in pairs])
    s_b = 1.0 / max(float(b[wet].std()), 1e-12)
    s_p = 1.0 / max(float(pp[wet].std()), 1e-12)
    s_out = max(float(dp[wet].std()), 1e-12)
    x = torch.stack([F, b * s_b, pp * s_p], dim=1)
    y = (dp / s_out)[:, None]
    m = wet[:, None].float()
    if objective == "residual":
        coef = torch.stack([torch.from_numpy(p["coef"].reshape(6, nz, ny, nx)).to(device) for p in pairs]).float()
        r0 = torch.stack([grid(p["b"]) for p in pairs])[:, None] * m - apply_operator(torch, pp[:, None], coef, m)
        s_r = max(float(r0[m > 0].std()), 1e-12)
    net = build_net(torch).to(device)
    opt = torch.optim.Adam(net.parameters(), lr=2e-3)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps)
    cx, cy, cz, edge, batch = min(40, nx), min(32, ny), min(32, nz), 4, 8
    gen = torch.Generator(device="cpu").manual_seed(seed)
    t0 = time.time()
    for step in range(steps):
        idx = torch.randint(0, len(pairs), (batch,), generator=gen)
        ox = torch.randint(0, nx - cx + 1, (batch,), generator=gen)
        oy = torch.randint(0, ny - cy + 1, (batch,), generator=gen)
        oz = torch.randint(0, nz - cz + 1, (batch,), generator=gen)
        xs = torch.stack([x[i, :, z:z + cz, yy:yy + cy, xx:xx + cx] for i, xx, yy, z in zip(idx, ox, oy, oz)])
        ys = torch.stack([y[i, :, z:z + cz, yy:yy + cy, xx:xx + cx] for i, xx, yy, z in zip(idx, ox, oy, oz)])
        ms = torch.stack([m[i, :, z:z + cz, yy:yy + cy, xx:xx + cx] for i, xx, yy, z in zip(idx, ox, oy, oz)])
        e = (slice(None), slice(None), slice(edge, cz - edge), slice(edge, cy - edge), slice(edge, cx - edge))
        pred = net(xs)
        if objective == "residual":
            cs = torch.stack([coef[i, :, z:z + cz, yy:yy + cy, xx:xx + cx] for i, xx, yy, z in zip(idx, ox, oy, oz)])
            rs = torch.stack([r0[i, :, z:z + cz, yy:yy + cy, xx:xx + cx] for i, xx, yy, z in zip(idx, ox, oy, oz)])
            res = (rs - apply_operator(torch, pred * s_out, cs, ms)) / s_r
            loss = (res[e] ** 2 * ms[e]).sum() / ms[e].sum().clamp(min=1.0)
        else:
            loss = ((pred - ys)[e] ** 2 * ms[e]).sum() / ms[e].sum().clamp(min=1.0)
        opt.zero_grad()
        loss.backward()
        opt.step()
        sched.step()
        if step % max(steps // 10, 1) == 0 or step == steps - 1:
            print(f"step {step}: masked MSE {loss.item():.4e} ({time.time() - t0:.1f} s)", flush=True)
    with torch.no_grad():  # whole-field score on the training pairs: fraction of the objective left
        if objective == "residual":
            resid = sum(float((((r0[i:i + 1] - apply_operator(torch, net(x[i:i + 1]) * s_out, coef[i:i + 1], m[i:i + 1])) ** 2)
                               * m[i:i + 1]).sum()) for i in range(len(pairs)))
            total = sum(float(((r0[i:i + 1] ** 2) * m[i:i + 1]).sum()) for i in range(len(pairs)))
        else:
            resid = sum(float((((net(x[i:i + 1]) - y[i:i + 1]) ** 2) * m[i:i + 1]).sum()) for i in range(len(pairs)))
            total = sum(float(((y[i:i + 1] ** 2) * m[i:i + 1]).sum()) for i in range(len(pairs)))
    convs = [mod for mod in net if isinstance(mod, torch.nn.Conv3d)]
    weights = [bf16_bits(c.weight.detach().permute(0, 2, 3, 4, 1).contiguous().cpu().numpy()) for c in convs]
    biases = [c.bias.detach().cpu().numpy().astype(np.float32) for c in convs]
    return weights, biases, (1.0, s_b, s_p), s_out, resid / max(total, 1e-30)


def train_cuda(bank, steps, seed=0, lr=2e-3, tensor=True):
    """The MSE objective trained with the library's own kernels (waves_net_train: forward, backward
    and Adam on the GPU) on the crops of a CropBank, the loss counted where the bank's mask is set;
    full-batch Adam for `steps` steps.  tensor: the tensor-core arithmetic (WAVES_NET_TENSOR), else
    the oracle's (WAVES_NET_EXACT)."""
    from waves_gb300.learned import net_gradients, net_train
    rng = np.random.default_rng(seed)
    xs, ys, ms, (s_b, s_p, s_out) = bank.batch()
    weights = [rng.normal(0.0, 1.0 / np.sqrt(27 * ci), size=(co, 27, ci)).astype(np.float32) * (0.1 if co == 1 else 1.0)
               for ci, co in CHANNELS]
    biases = [np.zeros(co, np.float32) for _, co in CHANNELS]
    t0 = time.time()
    weights, biases, hist = net_train(xs, ys, ms, weights, biases, steps, lr, tensor=tensor)
    print(f"cuda trainer ({'tensor' if tensor else 'exact'}): masked MSE {hist[0]:.4e} -> {hist[-1]:.4e} in {steps} steps ({time.time() - t0:.1f} s)", flush=True)
    total = float((ms * ys * ys).sum() / max(ms.sum(), 1.0))
    left, _, _, _ = net_gradients(xs, ys, ms, weights, biases, tensor=tensor)
    bits = [bf16_bits(w) for w in weights]
    return bits, biases, (1.0, s_b, s_p), s_out, left / max(total, 1e-30)


def evaluate(path, seeds, steps):
    weights, biases, iscale, oscale = load_model(path)
    rows = []
    for seed in seeds:
        row = {"seed": seed}
        for warm in (0, 1):
            cfg, a, T = beach(seed, warm)
            s = wg.WavesSolver(cfg)
            if warm:
                s.set_warm_start(weights, biases, iscale, oscale)
            s.request_time(1.0)
            s.run()
            c0 = s.control()
            import ctypes as C
            m_, p_, t_ = C.c_double(), C.c_double(), C.c_int64()
            s.lib.waves_timing(s.h, C.byref(m_), C.byref(p_), C.byref(t_), 1)
            s.request_steps(int(c0[2]) + steps)
            s.run()
            c1 = s.control()
            s.lib.waves_timing(s.h, C.byref(m_), C.byref(p_), C.byref(t_), 1)
            k = "learned" if warm else "plain"
            row[k] = {"iters_per_step": (c1[18] - c0[18]) / steps, "pressure_ms_per_step": p_.value / steps,
                      "warm_used": int(c1[102] - c0[102]), "trials": int(c1[32] - c0[32])}
            s.close()
        rows.append(row)
        print(json.dumps(row), flush=True)
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--pairs", type=int, default=40)
    ap.add_argument("--t0", type=float, default=1.0)
    ap.add_argument("--gap", type=float, default=0.1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--eval-seeds", type=int, default=2)
    ap.add_argument("--eval-steps", type=int, default=120)
    ap.add_argument("--out", default="model.npz")
    ap.add_argument("--objective", default="residual", choices=["residual", "mse"])
    ap.add_argument("--trainer", default="cuda", choices=["cuda", "torch"],
                    help="cuda: the library's own training kernels (MSE objective); torch: PyTorch")
    ap.add_argument("--crops", type=int, default=32,
                    help="--trainer cuda: training crops of 24^3 in all (cut from the pairs as they are captured)")
    ap.add_argument("--arithmetic", default="tensor", choices=["tensor", "exact"],
                    help="--trainer cuda: tensor-core implicit GEMM (tensor) or the oracle's order (exact)")
    args = ap.parse_args()
    cfg, _, _ = beach(1)
    seeds = range(1, args.seeds + 1)
    if args.trainer == "cuda":
        # crops cut as pairs are captured: the host keeps crops, never whole pairs
        args.objective = "mse"
        bank = CropBank(tuple(cfg.n), args.crops / max(args.seeds * args.pairs, 1))
        npairs = capture(seeds, args.pairs, args.t0, args.gap, sink=bank.add, with_coef=False)
        weights, biases, iscale, oscale, unexplained = train_cuda(bank, args.steps, 0,
                                                                  tensor=args.arithmetic == "tensor")
    else:
        import torch
        device = "cuda" if torch.cuda.is_available() else "cpu"
        pairs = capture(seeds, args.pairs, args.t0, args.gap)
        npairs = len(pairs)
        weights, biases, iscale, oscale, unexplained = train(pairs, tuple(cfg.n), args.steps, 0, device, args.objective)
    np.savez(args.out, **{f"w{l}": w for l, w in enumerate(weights)}, **{f"b{l}": b for l, b in enumerate(biases)},
             input_scale=np.array(iscale, np.float32), output_scale=np.float32(oscale),
             pairs=npairs, seeds=args.seeds, unexplained=unexplained)
    print(json.dumps({"pairs": npairs, "trainer": args.trainer, "objective": args.objective, "fraction_left": unexplained, "input_scale": iscale,
                      "output_scale": oscale, "out": args.out}), flush=True)
    if args.eval_seeds > 0:
        evaluate(args.out, range(101, 101 + args.eval_seeds), args.eval_steps)


if __name__ == "__main__":
    main()
