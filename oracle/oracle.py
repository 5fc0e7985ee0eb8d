"""ctypes front of the CPU oracle (``liboracle.so``) -- test infrastructure only.

Imported by ``tests/``, by ``__graft_entry__.smoke()`` as the checker and by
``bench.py``'s CPU baseline leg.  The product never imports this module.
"""

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

RULE_SUM_PRODUCT, RULE_NMS, RULE_OMS = 0, 1, 2
NOISE_LIBM, NOISE_CR = 0, 1
FRAME_DTYPE = np.dtype([("bit_errors", "<u4"), ("frame_error", "u1"), ("iterations", "u1"), ("pad", "<u2")])


def build(force=False):
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i32, i64, u64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_uint64, C.c_double
        L.or_rng_first.restype = u64
        L.or_rng_first.argtypes = [u64]
        L.or_fnv1a64.restype = u64
        L.or_fnv1a64.argtypes = [C.c_char_p, C.c_size_t]
        L.or_stream_draws.argtypes = [u64, u64, u64, u64, u64, vp]
        L.or_complex_gaussians.argtypes = [u64, u64, i32, vp, vp]
        L.or_code_new.restype = vp
        L.or_code_new.argtypes = [i32, i32, i32, i32, i32, i32, C.c_char_p, i32]
        L.or_code_from_alist.restype = vp
        L.or_code_from_alist.argtypes = [C.c_char_p, C.c_char_p, i32]
        L.or_code_from_rows.restype = vp
        L.or_code_from_rows.argtypes = [i32, i32, vp, vp, i32, C.c_char_p, i32]
        L.or_code_info_positions.argtypes = [vp, vp]
        L.or_link_trials.restype = i32
        L.or_link_trials.argtypes = [vp, i32, C.c_int64, i32, u64, u64, u64, u64, u64, C.c_double, i32, i32, vp, vp,
                                     vp]
        L.or_random_perm.argtypes = [i32, u64, vp]
        L.or_code_free.argtypes = [vp]
        L.or_code_info.argtypes = [vp, vp]
        L.or_code_bit_map.argtypes = [vp, vp]
        L.or_code_edges.argtypes = [vp, vp, vp]
        L.or_code_set_decoder.argtypes = [vp, i32, dbl, i32, i32]
        L.or_encode.argtypes = [vp, vp, vp]
        L.or_encode_full.argtypes = [vp, vp, vp]
        L.or_is_codeword.restype = i32
        L.or_is_codeword.argtypes = [vp, vp]
        L.or_bpsk_llr_batch.argtypes = [vp, u64, u64, u64, u64, i64, dbl, i32, vp, vp]
        L.or_code_set_demapper.argtypes = [vp, i32]
        L.or_demap_exact.argtypes = [i32, vp, vp, i64, dbl, vp]
        for f in (L.or_decode_f64, L.or_decode_f32):
            f.restype = i32
            f.argtypes = [vp, vp, vp, vp, vp]
        for f in (L.or_decode_llr_f64, L.or_decode_llr_f32):
            f.restype = i32
            f.argtypes = [vp, vp, vp]
        L.or_qam_points.restype = i32
        L.or_qam_points.argtypes = [i32, vp, vp, vp]
        L.or_demap_maxlog.argtypes = [i32, vp, vp, i64, dbl, vp]
        L.or_trial.restype = i32
        L.or_trial.argtypes = [vp, i32, u64, u64, u64, u64, dbl, i32, i32, vp, vp, vp]
        L.or_run_frames.restype = i32
        L.or_run_frames.argtypes = [vp, i32, u64, u64, u64, u64, u64, dbl, i32, i32, i32, vp]
        L.or_learned.restype = dbl
        L.or_learned.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp, i64, vp, vp, vp, i32]
        L.or_learned_f32.restype = dbl
        L.or_learned_f32.argtypes = [vp, i32, i32, i32, vp, vp, vp, vp, i64, vp, vp, vp, i32]
        L.or_learned_num_weights.restype = i64
        L.or_learned_num_weights.argtypes = [vp, i32, i32]
        L.or_bpsk_frame.restype = i32
        L.or_bpsk_frame.argtypes = [vp, u64, u64, u64, u64, dbl, vp]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def fnv1a64(name):
    b = name.encode() if isinstance(name, str) else bytes(name)
    return lib().or_fnv1a64(b, len(b))


def rng_first(seed):
    return lib().or_rng_first(seed)


def stream_draws(seed, name_hash, cond, trial, n):
    out = np.zeros(n, np.uint64)
    lib().or_stream_draws(seed, name_hash, cond, trial, n, _p(out))
    return out


def complex_gaussians(seed, n, mode=NOISE_LIBM):
    re, im = np.zeros(n), np.zeros(n)
    lib().or_complex_gaussians(seed, n, mode, _p(re), _p(im))
    return re, im


def random_perm(n, seed):
    """Interleaver::random(n, seed).perm()"""
    out = np.zeros(n, np.int32)
    lib().or_random_perm(n, seed, _p(out))
    return out


def qam(m):
    re, im, lm = np.zeros(m), np.zeros(m), C.c_double()
    if lib().or_qam_points(m, _p(re), _p(im), C.byref(lm)) != 0:
        raise ValueError(f"no square QAM of order {m}")
    return re + 1j * im, lm.value


def demap_maxlog(m, y, sigma2):
    y = np.ascontiguousarray(y, np.complex128)
    yr, yi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    out = np.zeros(len(y) * (m.bit_length() - 1))
    lib().or_demap_maxlog(m, _p(yr), _p(yi), len(y), sigma2, _p(out))
    return out


def demap_exact(m, y, sigma2):
    y = np.ascontiguousarray(y, np.complex128)
    yr, yi = np.ascontiguousarray(y.real), np.ascontiguousarray(y.imag)
    out = np.zeros(len(y) * (m.bit_length() - 1))
    lib().or_demap_exact(m, _p(yr), _p(yi), len(y), sigma2, _p(out))
    return out


class Code:
    """The oracle's NrLdpc, or a generic LdpcCode read from an alist text or given by its
    rows (the encoder of from_rows, or of accumulate)."""

    def __init__(self, k_info=None, e=None, bg=0, z=0, rv=0, qm=1, alist=None, rows=None, n=None,
                 accumulate=False):
        err = C.create_string_buffer(256)
        if rows is not None:
            start = np.zeros(len(rows) + 1, np.int32)
            start[1:] = np.cumsum([len(r) for r in rows])
            flat = np.array([v for r in rows for v in r], np.int32)
            self.h = lib().or_code_from_rows(n, len(rows), _p(start), _p(flat), int(bool(accumulate)), err, 256)
        elif alist is not None:
            self.h = lib().or_code_from_alist(alist.encode(), err, 256)
        else:
            self.h = lib().or_code_new(k_info, e, bg, z, rv, qm, err, 256)
        if not self.h:
            raise ValueError(err.value.decode())
        info = np.zeros(9, np.int64)
        lib().or_code_info(self.h, _p(info))
        (self.bg, self.z, self.k_info, self.e, self.k, self.n_full, self.n_rows, self.edges, self.ils) = (
            int(x) for x in info)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_code_free(self.h)
            self.h = None

    def set_demapper(self, exact):
        lib().or_code_set_demapper(self.h, int(bool(exact)))
        return self

    def set_decoder(self, rule=RULE_NMS, alpha=0.75, layered=True, max_iterations=20):
        lib().or_code_set_decoder(self.h, rule, alpha, int(layered), max_iterations)
        return self

    def bit_map(self):
        out = np.zeros(self.e, np.int64)
        lib().or_code_bit_map(self.h, _p(out))
        return out

    def edges_list(self):
        r, v = np.zeros(self.edges, np.int32), np.zeros(self.edges, np.int32)
        lib().or_code_edges(self.h, _p(r), _p(v))
        return r, v

    def encode(self, info):
        info = np.ascontiguousarray(info, np.uint8)
        out = np.zeros(self.e, np.uint8)
        lib().or_encode(self.h, _p(info), _p(out))
        return out

    def info_positions(self):
        out = np.zeros(self.k, np.int32)
        lib().or_code_info_positions(self.h, _p(out))
        return out

    def link_trials(self, blocks, interleaver_seed, m, seed, name_hash, cond, first, n, ebn0_db, noise=NOISE_CR,
                    threads=0, want_llr=False, want_payload=False):
        """Trials of the spec link fec_encode -> map -> awgn_ebn0 -> demap -> fec_decode
        (interleaver_seed None: no interleaver): counts [n][7] = raw errors, raw bits,
        coded errors, coded bits, block errors, blocks, iterations; optionally the
        deinterleaved LLRs and the payload bits."""
        out = np.zeros((n, 7), np.int64)
        llr = np.zeros((n, blocks * self.n_full)) if want_llr else None
        pay = np.zeros((n, blocks * self.k), np.uint8) if want_payload else None
        il = -1 if interleaver_seed is None else int(interleaver_seed)
        st = lib().or_link_trials(self.h, blocks, il, m, seed, name_hash, cond, first, n, ebn0_db, noise, threads,
                                  _p(out), _p(llr), _p(pay))
        if st != 0:
            raise ValueError(f"modulation order {m}")
        return out, llr, pay

    def encode_full(self, u):
        u = np.ascontiguousarray(u, np.uint8)
        out = np.zeros(self.n_full, np.uint8)
        lib().or_encode_full(self.h, _p(u), _p(out))
        return out

    def is_codeword(self, cw):
        return bool(lib().or_is_codeword(self.h, _p(np.ascontiguousarray(cw, np.uint8))))

    def decode(self, llr, precision="f64", want_app=False, want_post=False):
        """(bits, iterations, app, post) of NrLdpc::decode_block / app_into."""
        dt = np.float64 if precision == "f64" else np.float32
        llr = np.ascontiguousarray(llr, dt)
        bits = np.zeros(self.k_info, np.uint8)
        app = np.zeros(self.k_info, dt) if want_app else None
        post = np.zeros(self.n_full, dt) if want_post else None
        f = lib().or_decode_f64 if precision == "f64" else lib().or_decode_f32
        it = f(self.h, _p(llr), _p(bits), _p(app), _p(post))
        return bits, it, app, post

    def decode_llr(self, full, precision="f64"):
        dt = np.float64 if precision == "f64" else np.float32
        full = np.ascontiguousarray(full, dt)
        post = np.zeros(self.n_full, dt)
        f = lib().or_decode_llr_f64 if precision == "f64" else lib().or_decode_llr_f32
        it = f(self.h, _p(full), _p(post))
        return post, it

    def trial(self, m, seed, name_hash, cond, frame, ebn0_db, precision=0, noise=NOISE_CR):
        info = np.zeros(self.k_info, np.uint8)
        llr = np.zeros(self.e, np.float64)
        res = np.zeros(3, np.uint32)
        rc = lib().or_trial(self.h, m, seed, name_hash, cond, frame, ebn0_db, precision, noise, _p(info), _p(llr),
                            _p(res))
        if rc:
            raise ValueError("bad modulation")
        return info, llr, res

    def run_frames(self, m, seed, name_hash, cond, first, n, ebn0_db, precision=0, noise=NOISE_CR, threads=0):
        out = np.zeros(n, FRAME_DTYPE)
        rc = lib().or_run_frames(self.h, m, seed, name_hash, cond, first, n, ebn0_db, precision, noise, threads,
                                 _p(out))
        if rc:
            raise ValueError("bad modulation")
        return out

    def learned(self, T, shared, alpha, beta, llr, cw, want_post=False, want_grad=False, multi=False,
                info_only=False, precision="f64"):
        """(mean loss, post [n x n_full] or None, (d alpha, d beta) or None) of the learned min-sum;
        info_only: the loss over the K' information bits instead of all n_full bits;
        precision "f32": the GPU's f32 arithmetic (same messages and argmins as the GPU)."""
        f32 = precision == "f32"
        rt = np.float32 if f32 else np.float64
        llr = np.ascontiguousarray(llr, rt).reshape(-1, self.e)
        cw = np.ascontiguousarray(cw, np.uint8).reshape(-1, self.n_full)
        n = llr.shape[0]
        alpha = np.ascontiguousarray(alpha, np.float64)
        beta = np.ascontiguousarray(beta, np.float64)
        post = np.zeros((n, self.n_full), rt) if want_post else None
        ga = np.zeros_like(alpha) if want_grad else None
        gb = np.zeros_like(beta) if want_grad else None
        fn = lib().or_learned_f32 if f32 else lib().or_learned
        loss = fn(self.h, T, int(shared), int(multi), _p(alpha), _p(beta), _p(llr), _p(cw), n, _p(post), _p(ga), _p(gb),
                  int(bool(info_only)))
        if ga is None:
            return loss, post, None
        return loss, post, ((ga, gb) if f32 else (ga / n, gb / n))

    def learned_num_weights(self, T, shared):
        return int(lib().or_learned_num_weights(self.h, T, int(shared)))

    def bpsk_llr(self, seed, name_hash, cond, first, n, noise_var, threads=None):
        """(codewords [n][n_full] u8, channel LLRs [n][n_full] f64) of bpsk_frame's frames."""
        cw = np.zeros((n, self.n_full), np.uint8)
        llr = np.zeros((n, self.n_full), np.float64)
        lib().or_bpsk_llr_batch(self.h, seed, name_hash, cond, first, n, noise_var, threads or os.cpu_count() or 1,
                                _p(cw), _p(llr))
        return cw, llr

    def decode_llr_many(self, full, precision="f64"):
        """decode_llr of every row: (posteriors, iterations)."""
        dt = np.float64 if precision == "f64" else np.float32
        full = np.ascontiguousarray(full, dt).reshape(-1, self.n_full)
        post = np.zeros_like(full)
        its = np.zeros(full.shape[0], np.int32)
        f = lib().or_decode_llr_f64 if precision == "f64" else lib().or_decode_llr_f32
        for i in range(full.shape[0]):
            its[i] = f(self.h, _p(full[i]), _p(post[i]))
        return post, its

    def bpsk_frame(self, seed, name_hash, cond, trial, noise_var):
        res = np.zeros(2, np.uint32)
        lib().or_bpsk_frame(self.h, seed, name_hash, cond, trial, noise_var, _p(res))
        return int(res[0]), int(res[1])
