"""Training and evaluation of the learned min-sum against the plain min-sum.

* :func:`train` -- Adam steps on frames the frame generator draws (Eb/N0 uniform in a
  range), with a learning rate decaying geometrically from ``lr0`` to ``lr1``;
* :func:`fer_curve` -- FER per Eb/N0 point, frames in batches until ``min_errors``
  frame errors or ``max_frames`` (the ``min_errors("fer", n).or(max_trials(m))`` rule of
  crates/com-sim/src/stopping.rs), both decoders on the same frames;
* :func:`snr_at` -- the Eb/N0 at which a curve crosses a target FER (log-linear
  interpolation between the two bracketing points);
* :func:`save` / :func:`load` -- weights and training steps as an ``.npz`` checkpoint.

``python com-rs_gb300/learned.py c4`` runs the small-code protocol: the learned decoder
at 10 iterations against the plain normalised min-sum at 10, 20 and 50 iterations over
Eb/N0 0:0.25:3 dB, and the distance in dB to the plain 20-iteration curve at FER 1e-3.
``... c5`` runs the weight-shared BG1 Z = 384 64-QAM protocol (8 iterations).
``python com-rs_gb300/learned.py campaign c5`` runs the committed C5 weights, the plain
decoder at 20 and at 8 iterations down to FER 1e-5 (:func:`floor_campaign`).
"""

import json
import math
import os
import sys
import time

import numpy as np


def train(net, steps, batch, ebn0_lo, ebn0_hi, lr0=3e-3, lr1=3e-4, seed=11, name="learned_train", modulation=4,
          multi_loss=True, log_every=0):
    """`steps` Adam steps; returns the per-step losses."""
    losses = []
    for s in range(steps):
        lr = lr0 * (lr1 / lr0) ** (s / max(1, steps - 1))
        losses.append(net.train_step(seed, name, batch, ebn0_lo, ebn0_hi, lr, modulation, multi_loss))
        if log_every and (s + 1) % log_every == 0:
            print(f"  step {s + 1}: loss {np.mean(losses[-log_every:]):.5f}, lr {lr:.2e}", flush=True)
    return losses


def fer_curve(run_frames, grid, min_errors=300, max_frames=2_000_000, batch=65536, seed=13, name="learned_eval",
              modulation=4):
    """[(Eb/N0, frame errors, frames, FER, mean iterations)] of `run_frames` (the
    run_frames method of an NrLdpc or a LearnedNms)."""
    out = []
    for c, eb in enumerate(grid):
        fe = n = it = 0
        while fe < min_errors and n < max_frames:
            k = min(batch, max_frames - n)
            r = run_frames(seed, name, c, n, k, eb, modulation)
            fe += int(r["frame_error"].sum())
            it += int(r["iterations"].sum(dtype="u8"))
            n += k
        out.append((eb, fe, n, fe / n, it / n))
    return out


def floor_campaign(run_frames, grid, floor=1e-5, min_errors=100, max_frames=100_000_000, batch=65536, seed=13,
                   name="learned_campaign", modulation=4, point_wall_s=None, log=None):
    """A campaign down to a target FER: the grid points in increasing Eb/N0, each run until
    `min_errors` frame errors or `max_frames` frames (min_errors("fer", n).or(max_trials(m)),
    crates/com-sim/src/stopping.rs:143-156), stopping after the first point whose FER is at
    or below `floor`.  `point_wall_s` bounds one point's wall time (such a point is marked
    truncated).  Returns [(Eb/N0, frame errors, frames, FER, mean iterations, truncated)]."""
    out = []
    for c, eb in enumerate(grid):
        fe = n = it = 0
        t0 = time.time()
        truncated = False
        while fe < min_errors and n < max_frames:
            if point_wall_s is not None and time.time() - t0 > point_wall_s:
                truncated = True
                break
            k = min(batch, max_frames - n)
            r = run_frames(seed, name, c, n, k, eb, modulation)
            fe += int(r["frame_error"].sum())
            it += int(r["iterations"].sum(dtype="u8"))
            n += k
        out.append((eb, fe, n, fe / n, it / n, truncated))
        if log:
            log(f"  {eb:.2f} dB: {fe} / {n} frames, FER {fe / n:.3e}, {it / n:.2f} iterations"
                f"{' (wall limit)' if truncated else ''} [{time.time() - t0:.1f} s]")
        if fe / n <= floor:
            break
    return out


def snr_at(curve, target):
    """Eb/N0 where the FER of `curve` falls to `target` (None if it does not cross)."""
    pts = [(p[0], p[3]) for p in curve if p[3] > 0]
    for (e0, f0), (e1, f1) in zip(pts, pts[1:]):
        if f0 >= target >= f1 and f0 > f1:
            t = (math.log10(f0) - math.log10(target)) / (math.log10(f0) - math.log10(f1))
            return e0 + t * (e1 - e0)
    return None


def save(net, path):
    a, b = net.weights()
    np.savez(path, alpha=a, beta=b, steps=np.int64(net.steps()), iterations=np.int64(net.iterations),
             shared=np.int64(net.shared))


def load(net, path):
    d = np.load(path)
    if int(d["iterations"]) != net.iterations or bool(d["shared"]) != net.shared:
        raise ValueError("the checkpoint is for another network layout")
    net.set_weights(d["alpha"], d["beta"])


PROTOCOLS = {
    # K', E, base graph, Z, modulation, iterations, shared, train range, eval grid
    "c4": dict(k=520, e=1040, bg=2, z=52, m=4, T=10, shared=True, lo=1.0, hi=3.0, steps=3000, batch=4096,
               grid=[0.25 * i for i in range(13)], plain=(10, 20, 50), min_errors=300, max_frames=4_000_000),
    # the configured grid 2:0.1:4 dB lies below this code's waterfall (about 6.3 dB at 20
    # iterations, 7 dB at 8: 64-QAM at rate 1/2 without a bit interleaver, max-log LLRs), so
    # FER = 1 there for every decoder; the network is trained and compared on the waterfall
    "c5": dict(k=8448, e=16896, bg=1, z=384, m=64, T=8, shared=True, lo=6.0, hi=7.5, steps=3200, batch=1024,
               grid=[6.0 + 0.1 * i for i in range(16)], plain=(8, 20), min_errors=100, max_frames=1_000_000,
               configured_grid=[2.0 + 0.1 * i for i in range(21)],
               # the campaign to FER 1e-5: 100 frame errors or 1e8 frames per point
               campaign_grid=[6.0 + 0.1 * i for i in range(21)], campaign_min_errors=100,
               campaign_max_frames=100_000_000),
}


def run_campaign(cb, name, weights_dir, floor=1e-5, point_wall_s=300.0, log=print):
    """The protocol's decoders (the learned one with its committed weights, the plain one at
    20 iterations and at the learned one's count) down to FER `floor` on its grid."""
    p = PROTOCOLS[name]

    def nr(it):
        return cb.NrLdpc(p["k"], p["e"], base_graph=p["bg"], lifting_size=p["z"], precision="f32", max_iterations=it)

    net = cb.LearnedNms(nr(p["T"]), p["T"], shared=p["shared"])
    load(net, os.path.join(weights_dir, f"learned_{name}.npz"))
    grid = p.get("campaign_grid", p["grid"])
    curves, t0 = {}, time.time()
    for key, run in ((f"learned_{p['T']}", net.run_frames), ("plain_20", nr(20).run_frames),
                     (f"plain_{p['T']}", nr(p["T"]).run_frames)):
        log(f"{key}:")
        curves[key] = floor_campaign(run, grid, floor, p.get("campaign_min_errors", 100),
                                     p.get("campaign_max_frames", 100_000_000), modulation=p["m"],
                                     point_wall_s=point_wall_s, log=log)
    report = {"protocol": name, "floor": floor, "grid": grid, "point_wall_s": point_wall_s, "curves": curves,
              "wall_s": time.time() - t0}
    for target in (1e-2, 1e-3, 1e-4, 1e-5):
        report[f"ebn0_at_fer_{target:g}"] = {k: snr_at(v, target) for k, v in curves.items()}
    return report


def run_protocol(cb, name, out_dir="."):
    p = PROTOCOLS[name]
    t0 = time.time()
    code = cb.NrLdpc(p["k"], p["e"], base_graph=p["bg"], lifting_size=p["z"], precision="f32",
                     max_iterations=p["T"])
    net = cb.LearnedNms(code, p["T"], shared=p["shared"])
    losses = train(net, p["steps"], p["batch"], p["lo"], p["hi"], modulation=p["m"], log_every=max(1, p["steps"] // 10))
    t_train = time.time() - t0
    save(net, os.path.join(out_dir, f"learned_{name}.npz"))
    curves = {f"learned_{p['T']}": fer_curve(net.run_frames, p["grid"], p["min_errors"], p["max_frames"],
                                            modulation=p["m"])}
    for it in p["plain"]:
        plain = cb.NrLdpc(p["k"], p["e"], base_graph=p["bg"], lifting_size=p["z"], precision="f32",
                          max_iterations=it)
        curves[f"plain_{it}"] = fer_curve(plain.run_frames, p["grid"], p["min_errors"], p["max_frames"],
                                          modulation=p["m"])
    if "configured_grid" in p:
        curves[f"learned_{p['T']}_configured_grid"] = fer_curve(net.run_frames, p["configured_grid"], p["min_errors"],
                                                                 65536, modulation=p["m"])
    report = {"protocol": name, "settings": {k: v for k, v in p.items() if "grid" not in k}, "train_s": t_train,
              "loss_first": float(np.mean(losses[:20])), "loss_last": float(np.mean(losses[-20:])),
              "curves": curves}
    for target in (1e-2, 1e-3):
        report[f"ebn0_at_fer_{target:g}"] = {k: snr_at(v, target) for k, v in curves.items()}
    report["wall_s"] = time.time() - t0
    return report


if __name__ == "__main__":
    import importlib

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    cbm = importlib.import_module("com-rs_gb300")
    if len(sys.argv) > 1 and sys.argv[1] == "campaign":
        proto = sys.argv[2] if len(sys.argv) > 2 else "c5"
        rep = run_campaign(cbm, proto, os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights"))
    else:
        rep = run_protocol(cbm, sys.argv[1] if len(sys.argv) > 1 else "c4", sys.argv[2] if len(sys.argv) > 2 else ".")
    print(json.dumps(rep))
