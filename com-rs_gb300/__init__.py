"""comrs_gb300 -- the com-rs BICM-LDPC Monte Carlo trial on one GB300.

Python front of ``libcomrs_gb300.so`` (C ABI: ``include/comrs_gb300.h``).  It mirrors
the reference's Python surface for this path:

* :class:`NrLdpc` -- ``comrs.NrLdpc(k, e, base_graph=, rv=, qm=, rule=, alpha=,
  max_iterations=, layered=)`` (bindings/com-py/src/fec/nr.rs:52-83) with ``encode`` /
  ``decode`` / ``app``, plus the explicit ``lifting_size`` and the GPU ``precision``;
* :meth:`NrLdpc.run_frames` -- the Monte Carlo frames of one condition, frame f drawn
  from ``stream(seed, name, condition, f)`` (crates/com-sim/src/runner.rs:435-447);
* :class:`Ldpc` -- the reference's generic ``LdpcCode`` decoder (any parity-check matrix,
  alist files, sum-product or min-sum, layered or flooding; crates/com-fec/src/ldpc.rs);
* :func:`run` -- a campaign over an Eb/N0 grid with the ``min_errors(...).or(max_trials)``
  stopping rule of com-sim (crates/com-sim/src/stopping.rs:64-265);
* :class:`Link` and :func:`run_spec` -- the link ``fec_encode -> map -> awgn_ebn0 ->
  demap -> fec_decode`` of a com-spec specification over a PEG code (specs/bicm_ldpc.yaml)
  and the campaign of such a specification.

The compute runs only in the CUDA library: there is no CPU fallback.  Importing works
without a GPU; creating a code object needs one.
"""

import ctypes as C
import os

import numpy as np

from .campaign import Grid, Stop, run  # noqa: F401
from .dvbs2 import Dvbs2Ldpc  # noqa: F401
from .ldpc import Ldpc, parse_alist  # noqa: F401
from .mix import MIX_ITEM_DTYPE, MixBatch, autotune, draw_mixed_batch  # noqa: F401
from .spec import LINK_DTYPE, Link, load_yaml, run_spec  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcomrs_gb300.so")

RULES = {"normalized_min_sum": 1, "min_sum": 1, "offset_min_sum": 2, "sum_product": 0}
PRECISIONS = {"f64": 0, "f32": 1}
FRAME_DTYPE = np.dtype([("bit_errors", "<u4"), ("frame_error", "u1"), ("iterations", "u1"), ("reserved", "<u2")])


class ComrsError(RuntimeError):
    """A non-zero status of the C ABI (``cb_status``), with the library's message."""

    KINDS = {-1: "Config", -2: "Shape", -3: "Numerical", -4: "Condition", -5: "Io", -6: "Cuda"}

    def __init__(self, status, message):
        self.status = status
        self.kind = self.KINDS.get(status, "Unknown")
        super().__init__(f"{self.kind}: {message}")


class _Desc(C.Structure):
    _fields_ = [("k_info", C.c_int32), ("e", C.c_int32), ("base_graph", C.c_int32), ("lifting_size", C.c_int32),
                ("rv", C.c_int32), ("qm", C.c_int32), ("rule", C.c_int32), ("alpha", C.c_double),
                ("layered", C.c_int32), ("max_iterations", C.c_int32), ("precision", C.c_int32),
                ("device", C.c_int32)]


# (name, restype, argtypes) of every symbol of include/comrs_gb300.h
_vp, _i32, _i64, _u64, _dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
SYMBOLS = [
    ("cb_version", C.c_char_p, []),
    ("cb_code_create", _i32, [C.POINTER(_Desc), C.POINTER(_vp)]),
    ("cb_code_destroy", None, [_vp]),
    ("cb_last_error", C.c_char_p, [_vp]),
    ("cb_code_set_demapper", _i32, [_vp, _i32]),
    ("cb_code_prepare", _i32, [_vp]),
    ("cb_code_info", _i32, [_vp, _vp]),
    ("cb_code_tables", _i32, [_vp, _vp, _vp]),
    ("cb_encode", _i32, [_vp, _vp, _i64, _vp]),
    ("cb_decode", _i32, [_vp, _vp, _i64, _vp, _vp, _vp]),
    ("cb_decode_device", _i32, [_vp, _vp, _i64, _vp, _vp, _vp, _vp]),
    ("cb_run_frames", _i32, [_vp, _i32, _u64, _u64, _u64, _u64, _i64, _dbl, _vp]),
    ("cb_generate_frames", _i32, [_vp, _i32, _u64, _u64, _u64, _u64, _i64, _dbl, _vp, _vp]),
    ("cb_run_frames_device", _i32, [_vp, _i32, _u64, _u64, _u64, _u64, _i64, _dbl, _vp, _vp]),
    ("cb_generate_frames_device", _i32, [_vp, _i32, _u64, _u64, _u64, _u64, _i64, _dbl, _vp, _vp, _vp]),
    ("cb_nms_create", _i32, [_vp, _i32, _i32, C.POINTER(_vp)]),
    ("cb_nms_destroy", None, [_vp]),
    ("cb_nms_info", _i32, [_vp, _vp]),
    ("cb_nms_get_weights", _i32, [_vp, _vp, _vp]),
    ("cb_nms_set_weights", _i32, [_vp, _vp, _vp]),
    ("cb_nms_forward", _i32, [_vp, _vp, _i64, _vp]),
    ("cb_nms_set_loss_bits", _i32, [_vp, _i32]),
    ("cb_nms_gradients", _i32, [_vp, _vp, _vp, _i64, _i32, _vp, _vp, C.POINTER(_dbl)]),
    ("cb_nms_train_step", _i32, [_vp, _i32, _u64, _u64, _i64, _dbl, _dbl, _dbl, _i32, C.POINTER(_dbl)]),
    ("cb_nms_decode", _i32, [_vp, _vp, _i64, _vp, _vp]),
    ("cb_nms_decode_device", _i32, [_vp, _vp, _i64, _vp, _vp, _vp]),
    ("cb_nms_run_frames", _i32, [_vp, _i32, _u64, _u64, _u64, _u64, _i64, _dbl, _vp]),
    ("cb_mix_create", _i32, [_vp, _i64, _u64, _u64, _dbl, _i32, _i32, C.POINTER(_vp)]),
    ("cb_mix_destroy", None, [_vp]),
    ("cb_mix_last_error", C.c_char_p, [_vp]),
    ("cb_mix_classes", _i32, [_vp, _i32, _vp, C.POINTER(_i32)]),
    ("cb_mix_set_rows_per_thread", _i32, [_vp, _i32, _i32]),
    ("cb_mix_run", _i32, [_vp, _u64, _vp]),
    ("cb_mix_time_decode", _i32, [_vp, _i32, _i32, C.POINTER(_dbl)]),
    ("cb_mix_frames", _i32, [_vp, _u64, _vp, _vp]),
    ("cb_decode_device_noalloc", _i32, [_vp, _vp, _i64, _vp, _vp, _vp]),
    ("cb_xoshiro_jump", _i32, [_vp, _u64, _vp]),
    ("cb_ldpc_create", _i32, [_i32, _i32, _vp, _vp, _i32, _dbl, _i32, _i32, _i32, _i32, C.POINTER(_vp)]),
    ("cb_ldpc_destroy", None, [_vp]),
    ("cb_ldpc_last_error", C.c_char_p, [_vp]),
    ("cb_ldpc_info", _i32, [_vp, _vp]),
    ("cb_ldpc_levels", _i32, [_vp, _vp, _vp]),
    ("cb_ldpc_decode", _i32, [_vp, _vp, _i64, _vp, _vp]),
    ("cb_ldpc_decode_device", _i32, [_vp, _vp, _i64, _vp, _vp, _vp]),
    ("cb_ldpc_set_decoder", _i32, [_vp, _i32, _dbl, _i32, _i32]),
    ("cb_ldpc_girth", _i32, [_vp, _vp]),
    ("cb_ldpc_set_encoder", _i32, [_vp, _i32, _vp, _vp]),
    ("cb_ldpc_encode", _i32, [_vp, _vp, _i64, _vp]),
    ("cb_ldpc_encode_device", _i32, [_vp, _vp, _i64, _vp, _vp]),
    ("cb_ldpc_peg", _i32, [_i32, _i32, _i32, _u64, _vp, _vp]),
    ("cb_link_create", _i32, [_vp, _i32, _i32, _i32, _u64, _i32, C.POINTER(_vp)]),
    ("cb_link_destroy", None, [_vp]),
    ("cb_link_last_error", C.c_char_p, [_vp]),
    ("cb_link_info", _i32, [_vp, _vp]),
    ("cb_link_interleaver", _i32, [_vp, _vp]),
    ("cb_link_run_trials", _i32, [_vp, _u64, _u64, _u64, _u64, _i64, _dbl, _vp]),
    ("cb_link_run_trials_device", _i32, [_vp, _u64, _u64, _u64, _u64, _i64, _dbl, _vp, _vp]),
    ("cb_link_generate", _i32, [_vp, _u64, _u64, _u64, _u64, _i64, _dbl, _vp, _vp, _vp]),
]

_lib = None


def lib():
    """The loaded CUDA library (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() or "
                              "python com-rs_gb300/build.py (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SYMBOLS:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _check(status, handle=None):
    if status != 0:
        msg = lib().cb_last_error(handle)
        raise ComrsError(status, msg.decode() if msg else "")


def fnv1a64(name):
    """FNV-1a 64 of a scenario name (crates/com-core/src/rng.rs:58-65)."""
    h = 0xCBF29CE484222325
    for b in name.encode() if isinstance(name, str) else bytes(name):
        h ^= b
        h = (h * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def version():
    return lib().cb_version().decode()


def xoshiro_jump(state, steps):
    """The xoshiro256** state after `steps` draws (Rng::state / Rng::from_state)."""
    s = np.ascontiguousarray(state, np.uint64)
    out = np.zeros(4, np.uint64)
    _check(lib().cb_xoshiro_jump(_p(s), steps, _p(out)))
    return out


class NrLdpc:
    """The 5G NR LDPC code of K' information bits rate-matched to E bits, on a GPU.

    Mirrors ``comrs.NrLdpc`` (bindings/com-py/src/fec/nr.rs:52-83); decoder defaults are
    those of the benchmark configurations (layered normalised min-sum, alpha 0.75, 20
    iterations).  ``precision`` is the arithmetic of LLRs and messages: ``"f64"`` (the
    reference's, bit-exact) or ``"f32"``.
    """

    def __init__(self, k, e, base_graph=None, rv=0, qm=1, rule="normalized_min_sum", alpha=0.75,
                 max_iterations=20, layered=True, lifting_size=None, precision="f64", device=0,
                 demapper="max_log"):
        rule_l = rule.lower()
        if rule_l not in RULES:
            raise ComrsError(-1, f"rule must be one of {sorted(RULES)}, got {rule!r}")
        if precision not in PRECISIONS:
            raise ComrsError(-1, f"precision must be 'f64' or 'f32', got {precision!r}")
        d = _Desc(k, e, base_graph or 0, lifting_size or 0, rv, qm, RULES[rule_l],
                  1.0 if rule_l == "min_sum" else float(alpha), int(bool(layered)), max_iterations,
                  PRECISIONS[precision], device)
        h = C.c_void_p()
        _check(lib().cb_code_create(C.byref(d), C.byref(h)))
        self._h = h
        info = np.zeros(16, np.int64)
        _check(lib().cb_code_info(h, _p(info)), h)
        (self.bg, self.z, self.k_info, self.e, self.k_sys, self.n_full, self.n_rows, self.edges, self.ils,
         self.max_degree, self.rv, self.qm, self.core_terms, self.map_is_offset, self.n_entries, _) = (
            int(x) for x in info)
        if demapper not in ("max_log", "exact"):
            raise ComrsError(-1, f"demapper must be 'max_log' or 'exact', got {demapper!r}")
        _check(lib().cb_code_set_demapper(h, int(demapper == "exact")), h)
        self.demapper = demapper
        self.precision = precision
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.rule, self.alpha, self.max_iterations = rule_l, alpha, max_iterations

    def prepare(self):
        """Compile this code's decoder for its lifting into the on-disk cache (no GPU needed)."""
        _check(lib().cb_code_prepare(self._h), self._h)

    DECODERS = {-1: "not yet on a device", 0: "generic layered", 1: "base-graph layered min-sum",
                2: "layered min-sum compiled for this lifting"}

    @property
    def decoder(self):
        """The decoder kernel this code runs (cb_code_info field 15), once it has been on a device."""
        info = np.zeros(16, np.int64)
        _check(lib().cb_code_info(self._h, _p(info)), self._h)
        return self.DECODERS[int(info[15])]

    def close(self):
        if getattr(self, "_h", None):
            lib().cb_code_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference accessors (nr/ldpc.rs:164-182)
    def base_graph(self):
        return self.bg

    def lifting_size(self):
        return self.z

    @property
    def k(self):
        return self.k_info

    @property
    def n(self):
        return self.e

    def tables(self):
        """(entries [n_entries x 3] = (layer, base column, shift), bit map [E])."""
        ent = np.zeros((self.n_entries, 3), np.int32)
        bm = np.zeros(self.e, np.int32)
        _check(lib().cb_code_tables(self._h, _p(ent), _p(bm)), self._h)
        return ent, bm

    def bit_map(self):
        return self.tables()[1]

    def encode(self, info):
        """BlockCode::encode_block of one block (K' bits) or of rows of blocks."""
        u = np.ascontiguousarray(info, np.uint8)
        single = u.ndim == 1
        u2 = u.reshape(-1, self.k_info)
        out = np.zeros((u2.shape[0], self.e), np.uint8)
        _check(lib().cb_encode(self._h, _p(u2), u2.shape[0], _p(out)), self._h)
        return out[0] if single else out

    def _decode(self, llr, want_bits=True, want_app=False, want_iters=True):
        x = np.ascontiguousarray(llr, self.dtype)
        single = x.ndim == 1
        x2 = x.reshape(-1, self.e)
        n = x2.shape[0]
        bits = np.zeros((n, (self.k_info + 7) // 8), np.uint8) if want_bits else None
        app = np.zeros((n, self.k_info), self.dtype) if want_app else None
        it = np.zeros(n, np.int32) if want_iters else None
        _check(lib().cb_decode(self._h, _p(x2), n, _p(bits), _p(app), _p(it)), self._h)
        if bits is not None:
            bits = np.unpackbits(bits, axis=1, bitorder="little")[:, :self.k_info]
        return single, bits, app, it

    def decode(self, llr):
        """BlockCode::decode_block: the K' hard decisions of E channel LLRs (rows batched)."""
        single, bits, _, _ = self._decode(llr)
        return bits[0] if single else bits

    def decode_full(self, llr):
        """(hard decisions, a posteriori LLRs of the K' info bits, iterations)."""
        single, bits, app, it = self._decode(llr, want_app=True)
        if single:
            return bits[0], app[0], int(it[0])
        return bits, app, it

    def app(self, llr):
        """SoftDecode::app: the a posteriori LLRs of the information bits."""
        return self.decode_full(llr)[1]

    def run_frames(self, seed, name, condition, first_frame, n_frames, ebn0_db, modulation=4):
        """Per-frame (bit_errors, frame_error, iterations) of frames [first, first + n)."""
        out = np.zeros(n_frames, FRAME_DTYPE)
        nh = fnv1a64(name) if isinstance(name, (str, bytes)) else int(name)
        _check(lib().cb_run_frames(self._h, modulation, seed, nh, condition, first_frame, n_frames, ebn0_db,
                                   _p(out)), self._h)
        return out

    def generate_frames(self, seed, name, condition, first_frame, n_frames, ebn0_db, modulation=4):
        """(channel LLRs [n x E], info bits [n x K']) exactly as run_frames draws them."""
        llr = np.zeros((n_frames, self.e), self.dtype)
        info = np.zeros((n_frames, self.k_info), np.uint8)
        nh = fnv1a64(name) if isinstance(name, (str, bytes)) else int(name)
        _check(lib().cb_generate_frames(self._h, modulation, seed, nh, condition, first_frame, n_frames, ebn0_db,
                                        _p(llr), _p(info)), self._h)
        return llr, info


class LearnedNms:
    """The learned (neural) min-sum on an f32 NrLdpc: per-iteration scales and offsets,
    one per lifted edge or, with ``shared``, one per base-graph edge; starts as the
    plain normalised min-sum (its fallback)."""

    def __init__(self, code, iterations, shared=False):
        if code.precision != "f32":
            raise ComrsError(-1, "the learned min-sum runs on an f32 code object")
        self.code = code
        h = C.c_void_p()
        _check(lib().cb_nms_create(code._h, iterations, int(bool(shared)), C.byref(h)), code._h)
        self._h = h
        info = np.zeros(4, np.int64)
        _check(lib().cb_nms_info(h, _p(info)))
        self.n_weights, self.iterations, self.shared = int(info[0]), int(info[1]), bool(info[2])

    def close(self):
        if getattr(self, "_h", None):
            lib().cb_nms_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def steps(self):
        info = np.zeros(4, np.int64)
        _check(lib().cb_nms_info(self._h, _p(info)))
        return int(info[3])

    def weights(self):
        a, b = np.zeros(self.n_weights, np.float32), np.zeros(self.n_weights, np.float32)
        _check(lib().cb_nms_get_weights(self._h, _p(a), _p(b)), self.code._h)
        return a, b

    def set_weights(self, alpha, beta):
        a = np.ascontiguousarray(alpha, np.float32)
        b = np.ascontiguousarray(beta, np.float32)
        if a.size != self.n_weights or b.size != self.n_weights:
            raise ComrsError(-2, f"{self.n_weights} scales and offsets expected")
        _check(lib().cb_nms_set_weights(self._h, _p(a), _p(b)), self.code._h)

    def forward(self, llr):
        x = np.ascontiguousarray(llr, np.float32).reshape(-1, self.code.e)
        post = np.zeros((x.shape[0], self.code.n_full), np.float32)
        _check(lib().cb_nms_forward(self._h, _p(x), x.shape[0], _p(post)), self.code._h)
        return post

    def decode(self, llr):
        """(posteriors [n x n_full], iterations) with the syndrome stop after each iteration."""
        x = np.ascontiguousarray(llr, np.float32).reshape(-1, self.code.e)
        post = np.zeros((x.shape[0], self.code.n_full), np.float32)
        its = np.zeros(x.shape[0], np.int32)
        _check(lib().cb_nms_decode(self._h, _p(x), x.shape[0], _p(post), _p(its)), self.code._h)
        return post, its

    def set_loss_bits(self, info_only):
        """The bits the training loss covers: all n_full codeword bits, or (info_only) the
        K' information bits."""
        _check(lib().cb_nms_set_loss_bits(self._h, int(bool(info_only))), self.code._h)

    def gradients(self, llr, cw, multi_loss=False):
        """(mean loss, d/d scales, d/d offsets) of frames of E LLRs against their n_full
        codeword bits.  multi_loss: 0 (False) the last output's loss, 1 (True) the mean over
        every iteration's output, 2 their mean weighted 2 (t + 1) / (T (T + 1))."""
        x = np.ascontiguousarray(llr, np.float32).reshape(-1, self.code.e)
        c = np.ascontiguousarray(cw, np.uint8).reshape(-1, self.code.n_full)
        ga, gb = np.zeros(self.n_weights, np.float32), np.zeros(self.n_weights, np.float32)
        loss = C.c_double()
        _check(lib().cb_nms_gradients(self._h, _p(x), _p(c), x.shape[0], int(multi_loss), _p(ga), _p(gb),
                                      C.byref(loss)),
               self.code._h)
        return loss.value, ga, gb

    def train_step(self, seed, name, batch, ebn0_lo, ebn0_hi, lr, modulation=4, multi_loss=True):
        loss = C.c_double()
        nh = fnv1a64(name) if isinstance(name, (str, bytes)) else int(name)
        _check(lib().cb_nms_train_step(self._h, modulation, seed, nh, batch, ebn0_lo, ebn0_hi, lr, int(multi_loss),
                                       C.byref(loss)),
               self.code._h)
        return loss.value

    def run_frames(self, seed, name, condition, first_frame, n_frames, ebn0_db, modulation=4):
        out = np.zeros(n_frames, FRAME_DTYPE)
        nh = fnv1a64(name) if isinstance(name, (str, bytes)) else int(name)
        _check(lib().cb_nms_run_frames(self._h, modulation, seed, nh, condition, first_frame, n_frames, ebn0_db,
                                       _p(out)), self.code._h)
        return out
