#!/usr/bin/env python
"""Decoded info Gbit/s of the BICM-LDPC Monte Carlo trial on GB300, and its CPU baseline.

Workload (one "step" = one launch batch): 5G NR LDPC base graph 1, Z = 384, K' = 8448,
E = 25344 (rate 1/3), Gray 16-QAM, AWGN at Eb/N0 in 0:0.25:2 dB, max-log LLRs, layered
normalised min-sum alpha = 0.75, at most 20 iterations with the syndrome stop, f32 LLRs
and messages, 8192 codewords per launch.  Step s runs grid point s mod 9 on the next
8192 frames of that condition; frame f of condition c is drawn from
stream(seed = 7, "bicm_ldpc_c2", c, f).  The stop rule of the campaign (500 frame errors
or 1e6 frames per point) ends every point of this grid after its first batch (FER ~ 1),
so 9 steps are the whole campaign.

--impl ours (default): `value` = device-timed throughput of the frame generator and
the decoder (inputs: the frames' streams; every launch writes 830 MB of LLRs, more than
L2); `e2e` = the same through the public C ABI call cb_run_frames with the per-frame
records returned to pinned host memory every step; `roofline` = the decoder kernel
against the measured HBM copy bandwidth.
--impl reference: the CPU oracle's restatement of the reference trial (f64, the
reference's libm noise) on all host cores, a bounded sample of frames per step.

--workload mix: the uneven mixed batch: 16,384 codewords, each of a base graph, lifting size
Z, rate, modulation and Eb/N0 drawn uniformly (BG {1, 2}, Z {16, 32, 64, 128, 208, 384},
R {1/3, 1/2, 2/3, 5/6}, QPSK to 256-QAM, 0 to 6 dB), f32, at most 25 iterations, generated
and decoded by one replayed CUDA graph with per-codeword early exit and work stealing;
rows per thread autotuned.  One step = one replay on the next frames of every item.

--workload learned (--protocol c5 or c4): decoded info Gbit/s at equal FER, neural vs plain
min-sum.  The learned min-sum with the weights the committed protocol trained
(com-rs_gb300/weights/, from `python com-rs_gb300/learned.py c5|c4`) runs at its FER 1e-3
Eb/N0; the plain min-sum at 20 iterations and at the learned decoder's iteration count
run at theirs (measured on the protocol's curves).  `value` is the learned decoder's.

--workload spec: the link of com-rs's specs/bicm_ldpc.yaml instead (fec_encode of a PEG
(1024, 512) code, 8 blocks per trial, random interleaver, Gray 16-QAM, awgn_ebn0, exact
LLRs, layered sum-product with 50 iterations, f64), Eb/N0 2.5:0.5:5 dB, `--trials` trials
per step; step s runs grid point s mod 6.  Same keys; the roofline is the generic
decoder kernel against HBM (it is FP64-bound: the sum-product rule's tanh and atanh).
"""

import argparse
import ctypes as C
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "decoded info Gbit/s at equal FER, neural vs plain min-sum; vs CPU Runner"
K_INFO, E, BG, Z, M = 8448, 25344, 1, 384, 16
GRID = [0.25 * i for i in range(9)]
SEED, NAME = 7, "bicm_ldpc_c2"
# algorithmic bytes of one decoded codeword: E f32 LLRs in, ceil(K'/8) decision bytes out,
# a 4-byte record (iteration count)
ALGO_BYTES = E * 4 + (K_INFO + 7) // 8 + 4
# DRAM bytes (read + write) of the decoder per codeword at 20 iterations, and the
# warp-instructions it issues per codeword and iteration, from one ncu capture of a
# 2048-codeword launch of the decoder compiled for this code's lifting
# (profiles/decode_c2_f32.md: 207,803,136 + 81,634,560 B, smsp__inst_executed.sum =
# 3,337,917,248); the persistent grid keeps the same 304 state slots at any batch, so both
# scale by codewords
DRAM_BYTES_PER_CODEWORD = (207_803_136 + 81_634_560) / 2048
WARP_INST_PER_CODEWORD_ITERATION = 3_337_917_248 / (2048 * 20)
# edges of the lifted graph (BG1's 316 entries x Z) and the layered min-sum's algorithmic
# operations per edge and iteration
N_EDGES = 316 * 384
OPS_PER_EDGE_ITERATION = 10
WORKLOAD = ("5G NR LDPC BG1 Z=384 K'=8448 E=25344 (rate 1/3), Gray 16-QAM, AWGN Eb/N0 0:0.25:2 dB, "
            "max-log LLRs, layered NMS alpha=0.75, <=20 iterations + syndrome stop, 8192 codewords/launch")
# a point at the code's waterfall (FER about 0.13; the grid above sits at FER 1)
WATERFALL_DB = 2.7


def c2_config(world, frames):
    """The workload description both arms print (the arithmetic type is the line's dtype)."""
    return {"workload": WORKLOAD, "codewords_per_launch": frames, "ebn0_db": GRID,
            "l2": "inputs larger than L2: each step writes and reads 830 MB of LLRs",
            "parallelism": f"dp{world} (disjoint frame ranges per GPU)"}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def read_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms during the timed region
    (the C2 bench's timed region lasts about 0.2 s)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.rows, self.proc = device, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def start_ranks(world, local_rank):
    """This process's GPU and, under torchrun, its NCCL process group: (dist or None,
    barrier(), max_over_ranks(x)).  barrier() also synchronises the device."""
    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return dist, barrier, max_over_ranks


def cpu_sample(steps, warmup, threads=0, budget_s=2.0):
    """The oracle's trial (f64, libm noise, as the reference) over all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    cores = threads or os.cpu_count()
    code = O.Code(K_INFO, E, bg=BG, z=Z).set_decoder(O.RULE_NMS, 0.75, True, 20)
    h = O.fnv1a64(NAME)
    # size the per-step sample from a first timing: about budget_s of work per step
    t0 = time.perf_counter()
    code.run_frames(M, SEED, h, 0, 0, cores, GRID[0], 0, O.NOISE_LIBM, cores)
    per = (time.perf_counter() - t0) / cores
    n = max(cores, int(budget_s / per / cores) * cores)
    for s in range(warmup):
        code.run_frames(M, SEED, h, s % 9, 10_000_000 + s * n, n, GRID[s % 9], 0, O.NOISE_LIBM, cores)
    total_t, frames, fe = 0.0, 0, 0
    for s in range(steps):
        t0 = time.perf_counter()
        r = code.run_frames(M, SEED, h, s % 9, (s // 9) * n, n, GRID[s % 9], 0, O.NOISE_LIBM, cores)
        total_t += time.perf_counter() - t0
        frames += n
        fe += int(r["frame_error"].sum())
    gbps = frames * K_INFO / total_t / 1e9
    return gbps, cores, n, frames, total_t, fe / frames


def run_reference(args, rank):
    if rank != 0:
        return
    gbps, cores, n, frames, t, fer = cpu_sample(args.steps, args.warmup)
    sample = (f"{n} frames per step ({frames} in {args.steps} steps, {t:.1f} s, FER {fer:.3f}) of the same "
              f"workload, one frame per Runner trial, f64 decoder and libm noise as the reference")
    line = {"impl": "reference", "metric": METRIC, "value": gbps, "unit": "Gbit/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": c2_config(args.gpus, args.frames),
            "cpu_baseline": {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port", "sample": sample,
                             "cpu_model": cpu_model()},
            "e2e": {"value": gbps, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    dist, barrier, max_over_ranks = start_ranks(world, local_rank)
    cb = importlib.import_module("com-rs_gb300")
    L = cb.lib()
    B = args.frames
    code = cb.NrLdpc(K_INFO, E, base_graph=BG, lifting_size=Z, precision="f32", device=local_rank)
    h = code._h
    nh = cb.fnv1a64(NAME)
    results = torch.empty(B * 8, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    def step(s):
        cond = s % 9
        first = (s // 9) * B * world + rank * B
        st = L.cb_run_frames_device(h, M, SEED, nh, cond, first, B, GRID[cond], C.c_void_p(results.data_ptr()), sp)
        if st:
            raise cb.ComrsError(st, L.cb_last_error(h).decode())

    for s in range(args.warmup):
        step(10_000 + s)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fer_acc, it_acc = [], []
    with ClockSampler(local_rank) as clocks:
        ev0.record(stream)
        for s in range(args.steps):
            step(s)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    rec = results.cpu().numpy().view(cb.FRAME_DTYPE)
    fer_acc.append(float(rec["frame_error"].mean()))
    it_acc.append(float(rec["iterations"].mean()))
    value = args.steps * B * world * K_INFO / (ms * 1e-3) / 1e9

    # roofline of the decoder kernel: LLRs already in HBM, CUDA events around its launch
    llr = torch.empty((B, E), dtype=torch.float32, device="cuda")
    info = torch.empty((B, (K_INFO + 31) // 32), dtype=torch.int32, device="cuda")
    bits = torch.empty((B, (K_INFO + 31) // 32), dtype=torch.int32, device="cuda")
    iters = torch.empty(B, dtype=torch.int32, device="cuda")
    dec_ms, gen_ms, dec_it = [], [], []
    for rep in range(4):
        cond = rep % 9
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        st = L.cb_generate_frames_device(h, M, SEED, nh, cond, 1_000_000 + rep * B, B, GRID[cond],
                                         C.c_void_p(llr.data_ptr()), C.c_void_p(info.data_ptr()), sp)
        e1.record(stream)
        st |= L.cb_decode_device(h, C.c_void_p(llr.data_ptr()), B, C.c_void_p(bits.data_ptr()), None,
                                 C.c_void_p(iters.data_ptr()), sp)
        e2.record(stream)
        torch.cuda.synchronize()
        if st:
            raise cb.ComrsError(st, L.cb_last_error(h).decode())
        if rep:  # the first repetition is a warm-up
            gen_ms.append(e0.elapsed_time(e1))
            dec_ms.append(e1.elapsed_time(e2))
            dec_it.append(float(iters.float().mean()))
    dec = float(np.mean(dec_ms))
    achieved = B * ALGO_BYTES / (dec * 1e-3) / 1e9
    peaks = read_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": B * DRAM_BYTES_PER_CODEWORD, "traffic_source": "ncu capture of 2048 codewords, scaled",
                "kernel": f"layered_nr_kernel<1, ...> (decoder: {code.decoder})",
                "algorithmic_bytes_per_launch": B * ALGO_BYTES, "launch_ms": dec,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                "generator_launch_ms": float(np.mean(gen_ms))}
    # the bound that does apply: instruction issue (one warp-instruction per cycle per SM
    # sub-partition, four per SM), at the clock sampled during the timed region
    props = torch.cuda.get_device_properties(local_rank)
    sm_hz = (clocks.summary().get("sm_mhz") or 2070.0) * 1e6
    issue_peak = props.multi_processor_count * 4 * sm_hz
    issue_achieved = WARP_INST_PER_CODEWORD_ITERATION * B * float(np.mean(dec_it)) / (dec * 1e-3)
    roofline["issue"] = {"achieved": issue_achieved, "peak": issue_peak, "unit": "warp-inst/s",
                         "frac": issue_achieved / issue_peak,
                         "source": "warp-instructions per codeword-iteration from an ncu capture of 2048 codewords"}
    # the algorithmic-ops fraction: 10 operations per edge and iteration of the layered
    # min-sum (subtraction, magnitude, two compare-selects, sign product, output choice,
    # scaling, sign, addition, syndrome bit), against the issue peak in thread-instructions
    ops_achieved = OPS_PER_EDGE_ITERATION * N_EDGES * B * float(np.mean(dec_it)) / (dec * 1e-3)
    roofline["ops"] = {"achieved": ops_achieved, "peak": 32 * issue_peak, "unit": "thread-op/s",
                       "frac": ops_achieved / (32 * issue_peak), "ops_per_edge_iteration": OPS_PER_EDGE_ITERATION,
                       "edges": N_EDGES}

    # end to end through the public C ABI: per-frame records to pinned host memory, on the
    # host clock over three times the device-timed steps (a window of about 0.4 s, so that
    # one host hiccup of a few milliseconds moves the rate by a few percent at most)
    host = torch.empty(B * 8, dtype=torch.uint8, pin_memory=True)
    out_p = C.c_void_p(host.data_ptr())
    for s in range(2):
        L.cb_run_frames(h, M, SEED, nh, s % 9, 2_000_000 + s * B, B, GRID[s % 9], out_p)
    barrier()
    e2e_steps = 3 * args.steps
    t0 = time.perf_counter()
    for s in range(e2e_steps):
        cond = s % 9
        first = (s // 9) * B * world + rank * B
        st = L.cb_run_frames(h, M, SEED, nh, cond, first, B, GRID[cond], out_p)
        if st:
            raise cb.ComrsError(st, L.cb_last_error(h).decode())
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": e2e_steps * B * world * K_INFO / e2e_s / 1e9, "unit": "Gbit/s", "h2d_bytes_per_step": 0,
           "d2h_bytes_per_step": B * 8, "steps": e2e_steps, "api": "cb_run_frames (host records)",
           "inputs": "the frames' streams (seed, name, condition, frame index) passed as arguments"}

    # the BlockCode drop-in end to end (NrLdpc::decode_block, nr/ldpc.rs:216-220): one step's
    # f32 LLRs in pinned host memory -> cb_decode -> packed decisions and iteration counts
    # in host memory; the copies both ways are inside the timed call
    llr_host = torch.empty((B, E), dtype=torch.float32, pin_memory=True)
    llr_host.copy_(llr)
    bits_host = torch.empty((B, (K_INFO + 7) // 8), dtype=torch.uint8, pin_memory=True)
    it_host = torch.empty(B, dtype=torch.int32, pin_memory=True)
    bc_args = (h, C.c_void_p(llr_host.data_ptr()), B, C.c_void_p(bits_host.data_ptr()), None,
               C.c_void_p(it_host.data_ptr()))
    st = L.cb_decode(*bc_args)
    barrier()
    t0 = time.perf_counter()
    for _ in range(3):
        st |= L.cb_decode(*bc_args)
    barrier()
    bc_s = max_over_ranks((time.perf_counter() - t0) / 3)
    if st:
        raise cb.ComrsError(st, L.cb_last_error(h).decode())
    e2e_blockcode = {"value": B * world * K_INFO / bc_s / 1e9, "unit": "Gbit/s", "h2d_bytes_per_step": B * E * 4,
                     "d2h_bytes_per_step": B * ((K_INFO + 7) // 8) + B * 4, "ms_per_step": bc_s * 1e3,
                     "api": "cb_decode (pinned host f32 LLRs in; host packed decisions and iteration counts out)",
                     "mean_iterations": float(it_host.float().mean())}

    # the same trial at the code's waterfall, where the syndrome stop and the FER matter
    wf = []
    for s in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.cb_run_frames_device(h, M, SEED, nh, 9, (s * world + rank) * B, B, WATERFALL_DB,
                                    C.c_void_p(results.data_ptr()), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if st:
            raise cb.ComrsError(st, L.cb_last_error(h).decode())
        r = results.cpu().numpy().view(cb.FRAME_DTYPE)
        if s:
            wf.append((max_over_ranks(e0.elapsed_time(e1)), r))
    wf_ms = float(np.mean([x[0] for x in wf]))
    wf_rec = np.concatenate([x[1] for x in wf])
    waterfall = {"ebn0_db": WATERFALL_DB, "value": B * world * K_INFO / (wf_ms * 1e-3) / 1e9, "unit": "Gbit/s",
                 "fer": float(wf_rec["frame_error"].mean()), "frame_errors": int(wf_rec["frame_error"].sum()),
                 "frames": int(len(wf_rec)) * world, "mean_iterations": float(wf_rec["iterations"].mean()),
                 "ms_per_step": wf_ms}

    # neural vs plain min-sum at equal FER (the metric's comparison), on the learned
    # decoder's own code (benchmark config 5) with the protocol's committed weights; 6 steps
    # of 8192 frames each (with 2 steps, a once-per-process cost of about 1 ms fell in the
    # learned decoder's timed region: 10.2 against 9.6 ms per step)
    decoders, _, _, _ = learned_decoders("c5", 6, 2, world, rank, local_rank, barrier, max_over_ranks)

    # the batched uneven mix (benchmark config 3) through its public API, so that the default
    # line carries it too (`--workload mix` measures it with its roofline and CPU baseline)
    mix = mix_summary(local_rank, rank, world, barrier, max_over_ranks)

    cpu = None
    if rank == 0 and not args.no_cpu:
        gbps, cores, n, frames, t, _ = cpu_sample(2, 0, budget_s=5.0)
        gbps1, _, n1, frames1, t1, _ = cpu_sample(1, 0, threads=1, budget_s=4.0)
        cpu = {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
               "sample": f"{frames} frames ({t:.1f} s) of the same workload, grid points 0 and 0.25 dB, f64 decoder "
                         f"and libm noise as the reference; one thread: {frames1} frames ({t1:.1f} s) at 0 dB",
               "value_1_thread": gbps1, "cpu_model": cpu_model()}
    if rank == 0:
        config = c2_config(world, B)
        config.update({"last_step_fer": fer_acc[-1], "last_step_mean_iterations": it_acc[-1],
                       "waterfall": waterfall, "decoders": decoders, "mix": mix})
        line = {"metric": METRIC, "value": value, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (Monte Carlo frames from seeded streams)",
                "config": config, "e2e": e2e, "e2e_blockcode": e2e_blockcode, "roofline": roofline,
                "cpu_baseline": cpu, "clocks": clocks.summary(), "gpu_launches": 2 * args.steps}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


SPEC_N, SPEC_K, SPEC_BLOCKS, SPEC_M = 1024, 512, 8, 16
SPEC_GRID = [2.5 + 0.5 * i for i in range(6)]
SPEC_SEED, SPEC_NAME = 6, "bicm_ldpc"
SPEC_METRIC = "decoded info Gbit/s of the bicm_ldpc specification's link; vs CPU Runner"
SPEC_WORKLOAD = ("specs/bicm_ldpc.yaml link: PEG(1024, 512) var degree 3 seed 1, 8 blocks per trial, random "
                 "interleaver, Gray 16-QAM, AWGN Eb/N0 2.5:0.5:5 dB, exact LLRs, layered sum-product <= 50 "
                 "iterations + syndrome stop, f64")
# algorithmic bytes of one decoded codeword through cb_ldpc_decode_device: n f64 LLRs in,
# n f64 posteriors out, a 4-byte iteration count
SPEC_ALGO_BYTES = SPEC_N * 8 * 2 + 4
# dram__bytes_read.sum + dram__bytes_write.sum of one f64 decode of 2048 trials at 2.5 dB
# (profiles/spec_link_sparse.md: 141,528,576 + 90,683,392 B)
SPEC_TRAFFIC = 141_528_576 + 90_683_392


def spec_cpu_sample(steps, warmup, threads=0, budget_s=2.0):
    """The oracle's spec link (f64, libm noise, as the reference) over all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    cb = importlib.import_module("com-rs_gb300")
    cores = threads or os.cpu_count()
    code = O.Code(rows=cb.ldpc.peg_rows(SPEC_N, SPEC_K), n=SPEC_N).set_decoder(O.RULE_SUM_PRODUCT, 0.8, True, 50)
    code.set_demapper(True)
    h = O.fnv1a64(SPEC_NAME)

    def trials(cond, first, n):
        return code.link_trials(SPEC_BLOCKS, 0, SPEC_M, SPEC_SEED, h, cond, first, n, SPEC_GRID[cond],
                                O.NOISE_LIBM, cores)[0]

    t0 = time.perf_counter()
    trials(0, 0, cores)
    per = (time.perf_counter() - t0) / cores
    n = max(cores, int(budget_s / per / cores) * cores)
    for s in range(warmup):
        trials(s % 6, 10_000_000 + s * n, n)
    total_t, done, be = 0.0, 0, 0
    for s in range(steps):
        t0 = time.perf_counter()
        out = trials(s % 6, (s // 6) * n, n)
        total_t += time.perf_counter() - t0
        done += n
        be += int(out[:, 4].sum())
    gbps = done * SPEC_BLOCKS * SPEC_K / total_t / 1e9
    return gbps, cores, n, done, total_t, be / (done * SPEC_BLOCKS)


def run_spec_reference(args, rank):
    if rank != 0:
        return
    gbps, cores, n, done, t, bler = spec_cpu_sample(args.steps, args.warmup)
    sample = (f"{n} trials per step ({done} in {args.steps} steps, {t:.1f} s) of the same link, f64 with libm "
              f"noise and libm tanh/atanh as the reference")
    line = {"impl": "reference", "metric": SPEC_METRIC, "value": gbps, "unit": "Gbit/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": SPEC_WORKLOAD, "trials_per_step": n, "bler": bler},
            "cpu_baseline": {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": gbps, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_spec_ours(args, rank, world, local_rank):
    import torch

    dist, barrier, max_over_ranks = start_ranks(world, local_rank)
    cb = importlib.import_module("com-rs_gb300")
    L = cb.lib()
    T = args.trials
    code = cb.Ldpc.peg(SPEC_N, SPEC_K, rule="sum_product", max_iterations=50, device=local_rank)
    link = cb.Link(code, SPEC_BLOCKS, SPEC_M, True, 0, "exact")
    nh = cb.fnv1a64(SPEC_NAME)
    rec = torch.empty(T * 16, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    def step(s):
        cond = s % 6
        first = (s // 6) * T * world + rank * T
        st = L.cb_link_run_trials_device(link._h, SPEC_SEED, nh, cond, first, T, SPEC_GRID[cond],
                                         C.c_void_p(rec.data_ptr()), sp)
        if st:
            raise cb.ComrsError(st, L.cb_link_last_error(link._h).decode())

    for s in range(args.warmup):
        step(10_000 + s)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        ev0.record(stream)
        for s in range(args.steps):
            step(s)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    last = rec.cpu().numpy().view(cb.LINK_DTYPE)
    value = args.steps * T * world * SPEC_BLOCKS * SPEC_K / (ms * 1e-3) / 1e9

    # the same link with an f32 decoder (the f64 LLRs rounded once to f32)
    code32 = cb.Ldpc.peg(SPEC_N, SPEC_K, rule="sum_product", max_iterations=50, precision="f32", device=local_rank)
    link32 = cb.Link(code32, SPEC_BLOCKS, SPEC_M, True, 0, "exact")
    st = 0
    for s in range(args.warmup):
        st |= L.cb_link_run_trials_device(link32._h, SPEC_SEED, nh, s % 6, 20_000_000 + s * T, T, SPEC_GRID[s % 6],
                                          C.c_void_p(rec.data_ptr()), sp)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for s in range(args.steps):
        cond = s % 6
        st |= L.cb_link_run_trials_device(link32._h, SPEC_SEED, nh, cond, (s // 6) * T * world + rank * T, T,
                                          SPEC_GRID[cond], C.c_void_p(rec.data_ptr()), sp)
    e1.record(stream)
    torch.cuda.synchronize()
    if st:
        raise cb.ComrsError(st, L.cb_link_last_error(link32._h).decode())
    ms32 = max_over_ranks(e0.elapsed_time(e1))
    f32 = {"value": args.steps * T * world * SPEC_BLOCKS * SPEC_K / (ms32 * 1e-3) / 1e9, "unit": "Gbit/s",
           "ms_per_step": ms32 / args.steps, "dtype": "f32 decoder on the f64 LLRs rounded once to f32"}
    link32.close()

    # roofline of the decoder kernel: one step's LLRs in HBM, CUDA events around the decode
    llr_h, _, _ = link.generate(SPEC_SEED, SPEC_NAME, 0, 3_000_000, T, SPEC_GRID[0])
    llr = torch.from_numpy(llr_h).cuda()
    post = torch.empty_like(llr)
    iters = torch.empty(T * SPEC_BLOCKS, dtype=torch.int32, device="cuda")
    dec_ms = []
    for rep in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = L.cb_ldpc_decode_device(code._h, C.c_void_p(llr.data_ptr()), T * SPEC_BLOCKS,
                                     C.c_void_p(post.data_ptr()), C.c_void_p(iters.data_ptr()), sp)
        e1.record(stream)
        torch.cuda.synchronize()
        if st:
            raise cb.ComrsError(st, L.cb_ldpc_last_error(code._h).decode())
        if rep:
            dec_ms.append(e0.elapsed_time(e1))
    dec = float(np.mean(dec_ms))
    achieved = T * SPEC_BLOCKS * SPEC_ALGO_BYTES / (dec * 1e-3) / 1e9
    peaks = read_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": SPEC_TRAFFIC, "traffic_source": "ncu capture of one f64 decode of 2048 trials at 2.5 dB "
                                                          "(bench.py --workload spec --profile-case --trials 2048)",
                "kernel": "sparse_group_kernel<double, sum-product, register rows> (generic decoder, several codewords "
                          "per CTA)",
                "algorithmic_bytes_per_launch": T * SPEC_BLOCKS * SPEC_ALGO_BYTES, "launch_ms": dec,
                "mean_iterations": float(iters.float().mean()),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                "note": "FP64-bound (tanh/atanh per edge), not HBM-bound"}

    # end to end through the public C ABI: records to pinned host memory
    host = torch.empty(T * 16, dtype=torch.uint8, pin_memory=True)
    out_p = C.c_void_p(host.data_ptr())
    L.cb_link_run_trials(link._h, SPEC_SEED, nh, 0, 4_000_000, T, SPEC_GRID[0], out_p)
    barrier()
    t0 = time.perf_counter()
    for s in range(args.steps):
        cond = s % 6
        first = (s // 6) * T * world + rank * T
        st = L.cb_link_run_trials(link._h, SPEC_SEED, nh, cond, first, T, SPEC_GRID[cond], out_p)
        if st:
            raise cb.ComrsError(st, L.cb_link_last_error(link._h).decode())
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e = {"value": args.steps * T * world * SPEC_BLOCKS * SPEC_K / e2e_s / 1e9, "unit": "Gbit/s",
           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": T * 16, "api": "cb_link_run_trials (host records)",
           "inputs": "the trials' streams (seed, name, condition, trial index) passed as arguments"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        gbps, cores, n, done, t, _ = spec_cpu_sample(2, 0, budget_s=5.0)
        cpu = {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
               "sample": f"{done} trials ({t:.1f} s) of the same link at 2.5 and 3 dB, f64 with libm noise and "
                         f"libm tanh/atanh as the reference"}
    if rank == 0:
        line = {"metric": SPEC_METRIC, "value": value, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (Monte Carlo trials from seeded streams)",
                "config": {"workload": SPEC_WORKLOAD, "trials_per_step": T, "codewords_per_step": T * SPEC_BLOCKS,
                           "ebn0_db": SPEC_GRID,
                           "l2": "inputs larger than L2: each step writes and reads 134 MB of f64 LLRs at 2048 trials",
                           "parallelism": f"dp{world} (disjoint trial ranges per GPU)",
                           "last_step_bler": float(last["block_errors"].sum()) / (T * SPEC_BLOCKS)},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks.summary(),
                "gpu_launches": 3 * args.steps, "f32_decoder": f32}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


MIX_N, MIX_ITEMS_SEED, MIX_SEED, MIX_NAME = 16384, 2024, 7, "bicm_ldpc_mix"
# dram__bytes_read.sum + dram__bytes_write.sum of the decode phase of one replay
# (profiles/mix_decode.md: 289,709,056 + 17,732,096 B)
MIX_TRAFFIC = 289_709_056 + 17_732_096
MIX_METRIC = "decoded info Gbit/s of the uneven mixed batch (one graph replay per step); vs CPU Runner"
MIX_WORKLOAD = ("16,384 codewords per replay, each: BG {1,2}, Z {16,32,64,128,208,384}, R {1/3,1/2,2/3,5/6}, "
                "Gray QPSK..256-QAM, Eb/N0 U[0,6] dB (item seed 2024); f32, layered NMS alpha=0.75, <=25 "
                "iterations with per-codeword early exit; one persistent decoder with work stealing, CUDA graph")


def mix_cpu_sample(budget_s, threads=0):
    """The oracle's trial (f64, libm noise) of the mixed batch's items, one frame each,
    over all host threads (the oracle releases the interpreter lock), for about
    budget_s seconds: (Gbit/s, cores, items, seconds)."""
    from concurrent.futures import ThreadPoolExecutor

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    cb = importlib.import_module("com-rs_gb300")
    items = cb.draw_mixed_batch(n=MIX_N, seed=MIX_ITEMS_SEED)
    cores = threads or os.cpu_count()
    h = O.fnv1a64(MIX_NAME)
    codes = {}

    def code_of(it):
        key = (int(it["base_graph"]), int(it["lifting_size"]), int(it["k_info"]), int(it["e"]))
        if key not in codes:
            codes[key] = O.Code(key[2], key[3], bg=key[0], z=key[1]).set_decoder(O.RULE_NMS, 0.75, True, 25)
        return codes[key]

    def one(i):
        it = items[i]
        code_of(it).trial(int(it["modulation_order"]), MIX_SEED, h, int(it["condition"]), int(it["frame"]),
                          float(it["ebn0_db"]), 0, O.NOISE_LIBM)
        return int(it["k_info"])

    for it in items:  # every code's host tables first, outside the timed sample
        code_of(it)
    done, bits, t0 = 0, 0, time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        while time.perf_counter() - t0 < budget_s and done < MIX_N:
            n = min(4 * cores, MIX_N - done)
            bits += sum(ex.map(one, range(done, done + n)))
            done += n
    t = time.perf_counter() - t0
    return bits / t / 1e9, cores, done, t


def mix_summary(local_rank, rank, world, barrier, max_over_ranks, replays=3):
    """The mixed batch's throughput for the default line: autotuned, two warm-up replays,
    then `replays` replays timed on the host clock (device work and the records), and the
    decode phase alone event-timed inside the library."""
    cb = importlib.import_module("com-rs_gb300")
    items = cb.draw_mixed_batch(n=MIX_N, seed=MIX_ITEMS_SEED)
    mix = cb.MixBatch(items, seed=MIX_SEED, name=MIX_NAME, max_iterations=25, device=local_rank)
    try:
        tuned = cb.autotune(mix, reps=2, cache=False)
        bits = int(items["k_info"].sum())
        for s in range(2):
            mix.run(epoch=20_000 + s)
        barrier()
        fer = []
        t0 = time.perf_counter()
        for s in range(replays):
            rec = mix.run(epoch=s * world + rank)
            fer.append(float(rec["frame_error"].mean()))
        barrier()
        wall = max_over_ranks(time.perf_counter() - t0)
        dec_ms = mix.time_decode(-1, reps=3)
    finally:
        mix.close()
    return {"workload": MIX_WORKLOAD, "value": replays * world * bits / wall / 1e9, "unit": "Gbit/s",
            "ms_per_replay": wall / replays * 1e3, "decode_phase_ms": dec_ms, "mean_fer": float(np.mean(fer)),
            "codewords_per_replay": MIX_N, "rows_per_thread": {str(z): v[0] for z, v in tuned.items()},
            "timing": "host clock around the synchronous replay call (cb_mix_run: generator, decoder, records)"}


def run_mix_reference(args, rank):
    if rank != 0:
        return
    gbps, cores, done, t = mix_cpu_sample(max(2.0, 3.0 * args.steps))
    line = {"impl": "reference", "metric": MIX_METRIC, "value": gbps, "unit": "Gbit/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": MIX_WORKLOAD, "items_sampled": done},
            "cpu_baseline": {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
                             "sample": f"the first {done} items of the batch, one frame each ({t:.1f} s), f64 decoder "
                                       f"and libm noise as the reference"},
            "e2e": {"value": gbps, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_mix_ours(args, rank, world, local_rank):
    import torch

    dist, barrier, max_over_ranks = start_ranks(world, local_rank)
    cb = importlib.import_module("com-rs_gb300")
    items = cb.draw_mixed_batch(n=MIX_N, seed=MIX_ITEMS_SEED)
    mix = cb.MixBatch(items, seed=MIX_SEED, name=MIX_NAME, max_iterations=25, device=local_rank)
    tuned = cb.autotune(mix, reps=2, cache=False)
    bits = int(items["k_info"].sum())

    for s in range(args.warmup):
        mix.run(epoch=10_000 + s)
    barrier()
    fer = []
    with ClockSampler(local_rank) as clocks:
        t0 = time.perf_counter()
        for s in range(args.steps):
            rec = mix.run(epoch=s * world + rank)
            fer.append(float(rec["frame_error"].mean()))
        barrier()
        wall = max_over_ranks(time.perf_counter() - t0)
    value = args.steps * world * bits / wall / 1e9
    # the decode phase alone, event-timed inside the library, against HBM
    dec_ms = mix.time_decode(-1, reps=3)
    algo = int((items["e"].astype(np.int64) * 4 + (items["k_info"].astype(np.int64) + 7) // 8 + 4).sum())
    peaks = read_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = algo / (dec_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": MIX_TRAFFIC, "traffic_source": "ncu capture of the decode phase of one replay of this "
                                                          "batch (bench.py --workload mix --profile-case)",
                "kernel": "mix_decode_kernel (decode phase of a replay)",
                "algorithmic_bytes_per_launch": algo, "launch_ms": dec_ms,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                "note": "issue-bound like the single-code decoder; the HBM fraction is the algorithmic-bytes one"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        gbps, cores, done, t = mix_cpu_sample(10.0)
        cpu = {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
               "sample": f"the first {done} items of the batch, one frame each ({t:.1f} s), f64 decoder and libm "
                         f"noise as the reference"}
    if rank == 0:
        e2e = {"value": value, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": MIX_N * 8,
               "api": "cb_mix_run (graph replay, records to the host)",
               "inputs": "the items' streams (seed, name, condition, frame + epoch x items)"}
        line = {"metric": MIX_METRIC, "value": value, "unit": "Gbit/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (Monte Carlo frames from seeded streams)",
                "config": {"workload": MIX_WORKLOAD, "codewords_per_step": MIX_N, "info_bits_per_step": bits,
                           "rows_per_thread": {str(z): v[0] for z, v in tuned.items()},
                           "timing": "host clock around the synchronous replay call (device work and the 128 KB "
                                     "of records); value and e2e are the same measurement",
                           "l2": f"inputs larger than L2: each replay writes and reads {algo / 1e6:.0f} MB of LLRs",
                           "parallelism": f"dp{world} (disjoint epochs per GPU)",
                           "mean_fer": float(np.mean(fer))},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks.summary(),
                "gpu_launches": 2 * args.steps}
        print(json.dumps(line), flush=True)
    mix.close()
    if dist:
        dist.destroy_process_group()


# the Eb/N0 (dB) of FER 1e-3 on the protocol's curves, for the learned decoder, the plain
# decoder at 20 iterations and the plain decoder at the learned one's iteration count
LEARNED_POINTS = {"c5": {"learned": 6.97, "plain_20": 6.51, "plain_T": 7.33},
                  "c4": {"learned": 2.17, "plain_20": 2.09, "plain_T": 2.35}}
LEARNED_FRAMES = {"c5": 8192, "c4": 65536}
# dram__bytes_read.sum + dram__bytes_write.sum of one decode of a step's frames
# (profiles/learned_decode_c5.md: 554,217,728 + 61,175,808 B; C4, the table-driven kernel: 272,915,712 +
# 2,977,024 B)
LEARNED_TRAFFIC = {"c5": 554_217_728 + 61_175_808, "c4": 272_915_712 + 2_977_024}
LEARNED_METRIC = "decoded info Gbit/s at equal FER (1e-3), neural vs plain min-sum; vs CPU Runner"


def learned_setup(proto):
    cb = importlib.import_module("com-rs_gb300")
    Lm = importlib.import_module("com-rs_gb300.learned")
    p = Lm.PROTOCOLS[proto]
    return cb, Lm, p


def learned_workload(p, proto):
    return (f"{proto}: BG{p['bg']} Z={p['z']} K'={p['k']} E={p['e']}, Gray {p['m']}-QAM; learned min-sum "
            f"({p['T']} iterations, weights shared per base edge, trained by the protocol) at its FER 1e-3 Eb/N0 "
            f"against plain NMS alpha=0.75 at 20 and at {p['T']} iterations at theirs; f32, syndrome stop")


def learned_cpu_sample(proto, budget_s, threads=0):
    """The oracle's plain 20-iteration decoder (f64, libm noise: the reference, which has
    no learned decoder) at its FER 1e-3 point, over all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build()
    _, _, p = learned_setup(proto)
    cores = threads or os.cpu_count()
    code = O.Code(p["k"], p["e"], bg=p["bg"], z=p["z"]).set_decoder(O.RULE_NMS, 0.75, True, 20)
    h = O.fnv1a64("learned_bench")
    eb = LEARNED_POINTS[proto]["plain_20"]
    t0 = time.perf_counter()
    code.run_frames(p["m"], 1, h, 0, 0, cores, eb, 0, O.NOISE_LIBM, cores)
    per = (time.perf_counter() - t0) / cores
    n = max(cores, int(budget_s / per / cores) * cores)
    t0 = time.perf_counter()
    r = code.run_frames(p["m"], 1, h, 0, cores, n, eb, 0, O.NOISE_LIBM, cores)
    t = time.perf_counter() - t0
    return n * p["k"] / t / 1e9, cores, n, t, float(r["frame_error"].mean())


def run_learned_reference(args, rank):
    if rank != 0:
        return
    _, _, p = learned_setup(args.protocol)
    gbps, cores, n, t, fer = learned_cpu_sample(args.protocol, max(2.0, 2.0 * args.steps))
    line = {"impl": "reference", "metric": LEARNED_METRIC, "value": gbps, "unit": "Gbit/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": learned_workload(p, args.protocol), "frames": n, "fer": fer},
            "cpu_baseline": {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
                             "sample": f"{n} frames ({t:.1f} s) of the plain 20-iteration decoder at its FER 1e-3 "
                                       f"point, f64 and libm noise as the reference (which has no learned decoder)"},
            "e2e": {"value": gbps, "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def learned_decoders(proto, steps, warmup, world, rank, local_rank, barrier, max_over_ranks, frames=None):
    """Neural vs plain min-sum at equal FER: the learned decoder (the protocol's committed
    weights) at its FER 1e-3 Eb/N0, the plain decoder at 20 iterations and at the learned
    one's iteration count at theirs.  Each runs `steps` batches through its public call
    (generation, decoding, records to the host), timed on the host clock.  Returns
    ({decoder: figures}, the clocks of the learned decoder's run, its code, its network)."""
    cb, Lm, p = learned_setup(proto)
    B = frames or LEARNED_FRAMES[proto]
    pts = LEARNED_POINTS[proto]

    def nr(it):
        return cb.NrLdpc(p["k"], p["e"], base_graph=p["bg"], lifting_size=p["z"], precision="f32",
                         max_iterations=it, device=local_rank)

    code = nr(p["T"])
    net = cb.LearnedNms(code, p["T"], shared=p["shared"])
    Lm.load(net, os.path.join(ROOT, "com-rs_gb300", "weights", f"learned_{proto}.npz"))
    decoders = {"learned": (net.run_frames, pts["learned"]), "plain_20": (nr(20).run_frames, pts["plain_20"]),
                f"plain_{p['T']}": (nr(p["T"]).run_frames, pts["plain_T"])}
    out, clocks_summary = {}, None
    for key, (run, eb) in decoders.items():
        for s in range(warmup):
            run(3, "learned_bench", 1, 10_000_000 + s * B, B, eb, p["m"])
        barrier()
        recs = []
        with ClockSampler(local_rank) as clocks:
            t0 = time.perf_counter()
            for s in range(steps):
                recs.append(run(3, "learned_bench", 0, (s * world + rank) * B, B, eb, p["m"]))
            barrier()
            wall = max_over_ranks(time.perf_counter() - t0)
        r = np.concatenate(recs)
        out[key] = {"value": steps * world * B * p["k"] / wall / 1e9, "unit": "Gbit/s", "ebn0_db": eb,
                    "fer": float(r["frame_error"].mean()), "frame_errors": int(r["frame_error"].sum()),
                    "frames": int(len(r)) * world, "mean_iterations": float(r["iterations"].mean()),
                    "ms_per_step": wall / steps * 1e3}
        if key == "learned":
            clocks_summary = clocks.summary()
    return out, clocks_summary, code, net


def run_learned_ours(args, rank, world, local_rank):
    import torch

    dist, barrier, max_over_ranks = start_ranks(world, local_rank)
    cb, Lm, p = learned_setup(args.protocol)
    B = LEARNED_FRAMES[args.protocol]
    pts = LEARNED_POINTS[args.protocol]
    out, clocks_summary, code, net = learned_decoders(args.protocol, args.steps, args.warmup, world, rank,
                                                      local_rank, barrier, max_over_ranks)
    lv = out["learned"]
    # roofline of the learned decoder kernel: one step's frames generated into HBM, then
    # cb_nms_decode_device timed with CUDA events on torch's stream (the LLRs exceed L2)
    llr = torch.empty((B, p["e"]), dtype=torch.float32, device=f"cuda:{local_rank}")
    info = torch.empty((B, (p["k"] + 31) // 32), dtype=torch.int32, device=f"cuda:{local_rank}")
    post = torch.empty((B, code.n_full), dtype=torch.float32, device=f"cuda:{local_rank}")
    its = torch.empty(B, dtype=torch.int32, device=f"cuda:{local_rank}")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = cb.lib()
    st = L.cb_generate_frames_device(code._h, p["m"], 3, cb.fnv1a64("learned_bench"), 0, 0, B, pts["learned"],
                                     C.c_void_p(llr.data_ptr()), C.c_void_p(info.data_ptr()), sp)
    dec = []
    for rep in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        st |= L.cb_nms_decode_device(net._h, C.c_void_p(llr.data_ptr()), B, C.c_void_p(post.data_ptr()),
                                     C.c_void_p(its.data_ptr()), sp)
        e1.record()
        torch.cuda.synchronize()
        if rep:
            dec.append(e0.elapsed_time(e1))
    if st:
        raise cb.ComrsError(st, L.cb_last_error(code._h).decode())
    dec_ms = float(np.mean(dec))
    algo = B * (p["e"] * 4 + (p["k"] + 7) // 8 + 4)
    peaks = read_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = algo / (dec_ms * 1e-3) / 1e9
    traffic = LEARNED_TRAFFIC.get(args.protocol)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_source": "ncu capture of one decode of this step's frames (bench.py --workload learned "
                                  "--profile-case)" if traffic else None,
                "kernel": "layered decoder with the learned weights (cb_nms_decode_device)",
                "algorithmic_bytes_per_launch": algo, "launch_ms": dec_ms,
                "launch_mean_iterations": float(its.float().mean()),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                "note": "issue-bound like the plain decoder; algorithmic bytes: E LLRs in, K' decided bits and "
                        "the iteration count out per frame"}
    cpu = None
    if rank == 0 and not args.no_cpu:
        gbps, cores, n, t, fer = learned_cpu_sample(args.protocol, 5.0)
        cpu = {"value": gbps, "unit": "Gbit/s", "cores": cores, "kind": "port",
               "sample": f"{n} frames ({t:.1f} s) of the plain 20-iteration decoder at its FER 1e-3 point (FER "
                         f"{fer:.1e}), f64 and libm noise as the reference (which has no learned decoder)"}
    if rank == 0:
        line = {"metric": LEARNED_METRIC, "value": lv["value"], "unit": "Gbit/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": lv["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (Monte Carlo frames from seeded streams)",
                "config": {"workload": learned_workload(p, args.protocol), "frames_per_step": B,
                           "l2": f"inputs larger than L2: each step writes and reads {B * p['e'] * 4 / 1e6:.0f} MB "
                                 f"of LLRs",
                           "decoders": out, "timing": "host clock around cb_nms_run_frames / cb_run_frames "
                                                       "(generation, decoding, records to the host)",
                           "parallelism": f"dp{world} (disjoint frame ranges per GPU)"},
                "e2e": {"value": lv["value"], "unit": "Gbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": B * 8,
                        "api": "cb_nms_run_frames (records to the host)"},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks_summary,
                "gpu_launches": 2 * -(-B // 16384) * args.steps}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_spec_profile_case(args):
    """The small case of the spec link for ncu: `trials` trials generated once at 2.5 dB,
    their codewords then decoded three times by the f64 and three times by the f32
    generic decoder."""
    import torch

    cb = importlib.import_module("com-rs_gb300")
    L = cb.lib()
    T = args.trials
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = {}
    for prec in ("f64", "f32"):
        code = cb.Ldpc.peg(SPEC_N, SPEC_K, rule="sum_product", max_iterations=50, precision=prec)
        link = cb.Link(code, SPEC_BLOCKS, SPEC_M, True, 0, "exact")
        llr_h, _, _ = link.generate(SPEC_SEED, SPEC_NAME, 0, 0, T, SPEC_GRID[0])
        llr = torch.from_numpy(llr_h if prec == "f64" else llr_h.astype(np.float32)).cuda()
        post = torch.empty_like(llr)
        iters = torch.empty(T * SPEC_BLOCKS, dtype=torch.int32, device="cuda")
        st = 0
        for _ in range(3):
            st |= L.cb_ldpc_decode_device(code._h, C.c_void_p(llr.data_ptr()), T * SPEC_BLOCKS,
                                          C.c_void_p(post.data_ptr()), C.c_void_p(iters.data_ptr()), sp)
        torch.cuda.synchronize()
        if st:
            raise cb.ComrsError(st, L.cb_ldpc_last_error(code._h).decode())
        out[prec] = float(iters.float().mean())
        link.close()
    print(json.dumps({"profile_case": "spec", "trials": T, "mean_iterations": out}))


def run_profile_case(args):
    """The small case the committed ncu summaries capture: `frames` C2 codewords generated
    once (Eb/N0 = 1 dB), then decoded three times, in --precision."""
    import torch

    cb = importlib.import_module("com-rs_gb300")
    L = cb.lib()
    n = args.frames
    code = cb.NrLdpc(K_INFO, E, base_graph=BG, lifting_size=Z, precision=args.precision)
    llr = torch.empty((n, E), dtype=torch.float32 if args.precision == "f32" else torch.float64, device="cuda")
    info = torch.empty((n, (K_INFO + 31) // 32), dtype=torch.int32, device="cuda")
    bits = torch.empty((n, (K_INFO + 31) // 32), dtype=torch.int32, device="cuda")
    iters = torch.empty(n, dtype=torch.int32, device="cuda")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.cb_generate_frames_device(code._h, M, SEED, cb.fnv1a64(NAME), 0, 0, n, 1.0, C.c_void_p(llr.data_ptr()),
                                     C.c_void_p(info.data_ptr()), sp)
    for _ in range(3):
        st |= L.cb_decode_device(code._h, C.c_void_p(llr.data_ptr()), n, C.c_void_p(bits.data_ptr()), None,
                                 C.c_void_p(iters.data_ptr()), sp)
    torch.cuda.synchronize()
    if st:
        raise cb.ComrsError(st, L.cb_last_error(code._h).decode())
    print(json.dumps({"profile_case": n, "mean_iterations": float(iters.float().mean())}))


def run_mix_profile_case(args):
    """The small case of the mixed batch for ncu: the bench's batch, rows per thread at
    their defaults, replayed three times (generator and decoder each time)."""
    cb = importlib.import_module("com-rs_gb300")
    items = cb.draw_mixed_batch(n=MIX_N, seed=MIX_ITEMS_SEED)
    mix = cb.MixBatch(items, seed=MIX_SEED, name=MIX_NAME, max_iterations=25, device=0)
    fer = [float(mix.run(epoch=s)["frame_error"].mean()) for s in range(3)]
    mix.close()
    print(json.dumps({"profile_case": "mix", "items": MIX_N, "fer": fer}))


def run_learned_profile_case(args):
    """The small case of the learned decoder for ncu: one step's frames of the protocol
    generated at the learned decoder's FER 1e-3 point, then decoded three times."""
    import torch

    cb, Lm, p = learned_setup(args.protocol)
    B = LEARNED_FRAMES[args.protocol]
    code = cb.NrLdpc(p["k"], p["e"], base_graph=p["bg"], lifting_size=p["z"], precision="f32",
                     max_iterations=p["T"])
    net = cb.LearnedNms(code, p["T"], shared=p["shared"])
    Lm.load(net, os.path.join(ROOT, "com-rs_gb300", "weights", f"learned_{args.protocol}.npz"))
    llr = torch.empty((B, p["e"]), dtype=torch.float32, device="cuda")
    info = torch.empty((B, (p["k"] + 31) // 32), dtype=torch.int32, device="cuda")
    its = torch.empty(B, dtype=torch.int32, device="cuda")
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = cb.lib()
    st = L.cb_generate_frames_device(code._h, p["m"], 3, cb.fnv1a64("learned_bench"), 0, 0, B,
                                     LEARNED_POINTS[args.protocol]["learned"], C.c_void_p(llr.data_ptr()),
                                     C.c_void_p(info.data_ptr()), sp)
    for _ in range(3):
        st |= L.cb_nms_decode_device(net._h, C.c_void_p(llr.data_ptr()), B, None, C.c_void_p(its.data_ptr()), sp)
    torch.cuda.synchronize()
    if st:
        raise cb.ComrsError(st, L.cb_last_error(code._h).decode())
    print(json.dumps({"profile_case": "learned", "protocol": args.protocol, "frames": B,
                      "mean_iterations": float(its.float().mean())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=9)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--frames", type=int, default=8192)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", choices=["c2", "mix", "learned", "spec"], default="c2",
                    help="c2: the NR trial (the headline); mix: the uneven mixed batch; learned: neural vs plain "
                         "min-sum at equal FER; spec: the link of specs/bicm_ldpc.yaml")
    ap.add_argument("--protocol", choices=["c5", "c4"], default="c5", help="the code of --workload learned")
    ap.add_argument("--trials", type=int, default=2048, help="trials per step of --workload spec")
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32", help="the decoder of the c2 profile case")
    ap.add_argument("--profile-case", action="store_true",
                    help="generate --frames C2 codewords (--workload spec: --trials trials; mix: the batch; "
                         "learned: one step's frames) and decode them three times (for ncu)")
    args = ap.parse_args()
    if args.profile_case:
        {"spec": run_spec_profile_case, "mix": run_mix_profile_case, "learned": run_learned_profile_case,
         "c2": run_profile_case}[args.workload](args)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.workload == "spec":
        if args.impl == "reference":
            run_spec_reference(args, rank)
        else:
            run_spec_ours(args, rank, world, local_rank)
    elif args.workload == "mix":
        if args.impl == "reference":
            run_mix_reference(args, rank)
        else:
            run_mix_ours(args, rank, world, local_rank)
    elif args.workload == "learned":
        if args.impl == "reference":
            run_learned_reference(args, rank)
        else:
            run_learned_ours(args, rank, world, local_rank)
    elif args.impl == "reference":
        run_reference(args, rank)
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
