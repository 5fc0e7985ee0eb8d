"""Mixed batches: thousands of codewords of uneven codes in one persistent launch.

* :func:`draw_mixed_batch` -- the items of an uneven mix: per codeword a base graph, a
  lifting size, a code rate, a modulation and an Eb/N0 drawn uniformly from a fixed
  seed (numpy's PCG64), K' = 22 Z or 10 Z, E = Qm ceil(K' / (R Qm)) capped at the
  circular buffer (the rate rule of the uneven-mix benchmark);
* :class:`MixBatch` -- the C ABI's cb_mix: generate and decode the batch by one
  replayed CUDA graph, records in the items' order;
* :func:`autotune` -- per lifting-size class, the lifted rows per thread (1 or 2)
  whose timed decode phase is fastest, cached per device and lifting size.
"""

import ctypes as C
import json
import os

import numpy as np

MIX_ITEM_DTYPE = np.dtype([("base_graph", "<i4"), ("lifting_size", "<i4"), ("k_info", "<i4"), ("e", "<i4"),
                           ("modulation_order", "<i4"), ("reserved", "<i4"), ("ebn0_db", "<f8"),
                           ("condition", "<u8"), ("frame", "<u8")])

RATES = ((1, 3), (1, 2), (2, 3), (5, 6))


def mix_e(bg, z, qm, rate):
    """E = Qm ceil(K' / (R Qm)) capped at the circular buffer N_cb = n_full - 2Z."""
    num, den = rate
    k = (22 if bg == 1 else 10) * z
    ncb = ((68 if bg == 1 else 52) - 2) * z
    e = qm * -(-(k * den) // (num * qm))
    return min(e, ncb - ncb % qm)


def draw_mixed_batch(n=16384, seed=2024, zs=(16, 32, 64, 128, 208, 384), mods=(4, 16, 64, 256),
                     ebn0=(0.0, 6.0), condition=0):
    rng = np.random.default_rng(seed)
    items = np.zeros(n, MIX_ITEM_DTYPE)
    bg = rng.integers(1, 3, n)
    z = np.asarray(zs)[rng.integers(0, len(zs), n)]
    r = rng.integers(0, len(RATES), n)
    m = np.asarray(mods)[rng.integers(0, len(mods), n)]
    items["base_graph"] = bg
    items["lifting_size"] = z
    items["k_info"] = np.where(bg == 1, 22, 10) * z
    items["e"] = [mix_e(int(b), int(zz), int(mm).bit_length() - 1, RATES[int(rr)]) for b, zz, mm, rr in
                  zip(bg, z, m, r)]
    items["modulation_order"] = m
    items["ebn0_db"] = rng.uniform(ebn0[0], ebn0[1], n)
    items["condition"] = condition
    items["frame"] = np.arange(n, dtype=np.uint64)
    return items


class MixBatch:
    def __init__(self, items, seed=7, name="bicm_ldpc_mix", alpha=0.75, max_iterations=25, device=0):
        from . import ComrsError, fnv1a64, lib

        self._lib, self._err = lib(), ComrsError
        self.items = np.ascontiguousarray(items, MIX_ITEM_DTYPE)
        self.n = len(self.items)
        nh = fnv1a64(name) if isinstance(name, (str, bytes)) else int(name)
        h = C.c_void_p()
        st = self._lib.cb_mix_create(C.c_void_p(self.items.ctypes.data), self.n, seed, nh, alpha, max_iterations,
                                     device, C.byref(h))
        if st:
            raise ComrsError(st, self._lib.cb_mix_last_error(None).decode())
        self._h = h

    def _check(self, st):
        if st:
            raise self._err(st, self._lib.cb_mix_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cb_mix_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def classes(self):
        """[dict(z, count, rows_per_thread, slots, slot_threads, smem_per_slot, grid, first)]"""
        n = C.c_int32()
        self._check(self._lib.cb_mix_classes(self._h, 0, None, C.byref(n)))
        info = np.zeros((n.value, 8), np.int64)
        self._check(self._lib.cb_mix_classes(self._h, n.value, C.c_void_p(info.ctypes.data), C.byref(n)))
        keys = ("z", "count", "rows_per_thread", "slots", "slot_threads", "smem_per_slot", "grid", "first")
        return [dict(zip(keys, (int(v) for v in row))) for row in info]

    def set_rows_per_thread(self, cls, rho):
        self._check(self._lib.cb_mix_set_rows_per_thread(self._h, cls, rho))

    def run(self, epoch=0):
        from . import FRAME_DTYPE

        out = np.zeros(self.n, FRAME_DTYPE)
        self._check(self._lib.cb_mix_run(self._h, epoch, C.c_void_p(out.ctypes.data)))
        return out

    def frames(self, epoch=0):
        """The generator's frames at `epoch`: ([E_i f32 LLRs], [K'_i info bits]) per item, in
        the items' order (the LLRs the decoder reads)."""
        e = self.items["e"].astype(np.int64)
        k = self.items["k_info"].astype(np.int64)
        llr = np.zeros(int(e.sum()), np.float32)
        info = np.zeros(int(k.sum()), np.uint8)
        self._check(self._lib.cb_mix_frames(self._h, epoch, C.c_void_p(llr.ctypes.data), C.c_void_p(info.ctypes.data)))
        return np.split(llr, np.cumsum(e)[:-1]), np.split(info, np.cumsum(k)[:-1])

    def time_decode(self, cls=-1, reps=3):
        ms = C.c_double()
        self._check(self._lib.cb_mix_time_decode(self._h, cls, reps, C.byref(ms)))
        return ms.value


# the rows per thread the mixed decoder is compiled for
ROWS_PER_THREAD = (1, 2)


def _cache_path():
    base = os.environ.get("COMRS_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "comrs_gb300")
    return os.path.join(base, "mix_autotune.json")


def autotune(batch, reps=3, cache=True, device_name=None):
    """Choose rows per thread per class by timing the decode phase; returns
    {z: (rows per thread, {candidate: ms})}.  Cached per device and lifting size."""
    if device_name is None:
        try:
            import torch

            device_name = torch.cuda.get_device_name()
        except Exception:
            device_name = "unknown"
    path = _cache_path()
    store = {}
    if cache and os.path.exists(path):
        try:
            store = json.load(open(path))
        except Exception:
            store = {}
    dev = store.setdefault(device_name, {})
    chosen = {}
    for k, cls in enumerate(batch.classes()):
        key = str(cls["z"])
        if cache and key in dev and dev[key].get("rows_per_thread") in ROWS_PER_THREAD:
            rho, times = dev[key]["rows_per_thread"], dev[key]["ms"]
        else:
            times = {}
            for rho in ROWS_PER_THREAD:
                try:
                    batch.set_rows_per_thread(k, rho)
                except Exception:
                    continue
                times[rho] = batch.time_decode(k, reps) / max(1, cls["count"])
            rho = min(times, key=times.get)
            dev[key] = {"rows_per_thread": rho, "ms": times}
        batch.set_rows_per_thread(k, rho)
        chosen[cls["z"]] = (rho, times)
    if cache:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        json.dump(store, open(path, "w"), indent=1)
    return chosen
