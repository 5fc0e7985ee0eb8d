"""Generic sparse LDPC codes on the GPU: the reference's ``LdpcCode`` (crates/com-fec/src/ldpc.rs)
with the surface of its Python class (bindings/com-py/src/fec/ldpc_code.rs).

* :func:`parse_alist` -- MacKay's ``alist`` format with the checks of the reference's
  parser (ldpc.rs:638-741): comments after ``#``, lists padded with zeros or not,
  degrees that reach their declared maxima, 1-based indices in range and not repeated,
  column and row lists that agree.  It returns ``(n, rows)``, rows in file order.
* :class:`Ldpc` -- a code of ``n`` variables and the given rows.  Constructors:
  ``Ldpc(n, rows)`` (``LdpcCode::from_rows``, ldpc.rs:216-231), :meth:`Ldpc.peg`
  (progressive edge growth, ldpc.rs:289-313), :meth:`Ldpc.accumulate` (IRA codes,
  ldpc.rs:233-256), :meth:`Ldpc.from_alist` / :meth:`Ldpc.from_alist_file`
  (ldpc.rs:350-380).  Decoded on the GPU by ``cb_ldpc_decode`` with the settings of
  ``LdpcDecoder`` (ldpc.rs:165-172; :meth:`Ldpc.set_decoder`): rule ``sum_product``,
  ``min_sum``, ``normalized_min_sum`` or ``offset_min_sum`` (``CheckRule::from_name``,
  ldpc.rs:104-113), layered or flooding schedule, maximum iterations.  Encoded on the
  GPU by ``cb_ldpc_encode`` (``encode_block``, ldpc.rs:753-791).

The GF(2) elimination that gives ``k``, the information positions and the encoder of
``from_rows`` runs on first use of any of them (``k``, ``rate``, ``info_positions``,
``encode``, ``decode``), not at construction as in the reference: a code without
information bits raises there.  There is no CPU decoder or encoder here: without the
CUDA library the calls raise.
"""

import ctypes as C

import numpy as np

# the reference's defaults (ldpc.rs:16-29)
DEFAULT_RULE = "sum_product"
DEFAULT_ALPHA = 0.8
DEFAULT_LAYERED = True
DEFAULT_MAX_ITERATIONS = 50


def _alist_numbers(text):
    out = []
    for ln, line in enumerate(text.splitlines()):
        for tok in line.split("#", 1)[0].split():
            if not tok.isdigit():
                raise ValueError(f"alist: line {ln + 1}: {tok!r} is not a number")
            out.append(int(tok))
    return out


def _alist_lists(rest, pos, degrees, width, bound, what):
    out = []
    for i, d in enumerate(degrees):
        n = width if width is not None else d
        entries = rest[pos:pos + n]
        pos += n
        ones, zeros = entries[:d], entries[d:]
        if any(z != 0 for z in zeros):
            raise ValueError(f"alist: {what} {i + 1}: more entries than its degree {d}")
        lst = []
        for e in ones:
            if e == 0 or e > bound:
                raise ValueError(f"alist: {what} {i + 1}: the index {e} is outside 1 to {bound}")
            if e - 1 in lst:
                raise ValueError(f"alist: {what} {i + 1}: the index {e} is repeated")
            lst.append(e - 1)
        out.append(lst)
    return out, pos


def parse_alist(text):
    """(n, rows) of an alist text; ValueError for a malformed file."""
    nums = iter(_alist_numbers(text))

    def nxt(what):
        try:
            return next(nums)
        except StopIteration:
            raise ValueError(f"alist: the file ends before {what}") from None

    n, m = nxt("the number of columns"), nxt("the number of rows")
    if n == 0 or m == 0:
        raise ValueError(f"alist: a matrix of {m} × {n}")
    max_col, max_row = nxt("the largest column degree"), nxt("the largest row degree")
    col_deg = [nxt("the column degrees") for _ in range(n)]
    row_deg = [nxt("the row degrees") for _ in range(m)]
    for deg, mx, what in ((col_deg, max_col, "column"), (row_deg, max_row, "row")):
        if any(d > mx for d in deg) or max(deg) != mx:
            raise ValueError(f"alist: the {what} degrees do not have the maximum {mx}")
    edges = sum(col_deg)
    if sum(row_deg) != edges:
        raise ValueError(f"alist: the column degrees count {edges} ones, the row degrees {sum(row_deg)}")
    rest = list(nums)
    if len(rest) == n * max_col + m * max_row:
        padded = True
    elif len(rest) == 2 * edges:
        padded = False
    else:
        raise ValueError(f"alist: {len(rest)} numbers after the degrees: {n * max_col + m * max_row} with zero "
                         f"padding or {2 * edges} without")
    cols, pos = _alist_lists(rest, 0, col_deg, max_col if padded else None, m, "column")
    rows, _ = _alist_lists(rest, pos, row_deg, max_row if padded else None, n, "row")
    for c, col in enumerate(cols):
        for r in col:
            if c not in rows[r]:
                raise ValueError(f"alist: column {c + 1} lists row {r + 1} but row {r + 1} does not list it")
    return n, rows


ENCODERS = {"sums": 0, "accumulate": 1}

# LdpcCode::peg defaults (ldpc.rs:86-88)
DEFAULT_VAR_DEGREE = 3
DEFAULT_PEG_SEED = 1


def _rule(rule):
    """The rule's name, as CheckRule::from_name reads it (case-insensitive)."""
    from . import ComrsError

    name = rule.lower() if isinstance(rule, str) else rule
    if name not in ("sum_product", "min_sum", "normalized_min_sum", "offset_min_sum"):
        raise ComrsError(-1, "rule must be sum_product, min_sum, normalized_min_sum or offset_min_sum, "
                             f"got {rule!r}")
    return name


def peg_rows(n, k, var_degree=DEFAULT_VAR_DEGREE, seed=DEFAULT_PEG_SEED):
    """The rows of ``LdpcCode::peg(n, k, var_degree, seed)`` (ldpc.rs:289-313), built by
    ``cb_ldpc_peg`` on the host: check c lists its variables in the order they were linked."""
    from . import ComrsError, lib

    L = lib()
    n, k, var_degree = int(n), int(k), int(var_degree)
    m = n - k
    start = np.zeros(max(m, 0) + 1, np.int32)
    vars_ = np.zeros(max(n * var_degree, 1), np.int32)
    st = L.cb_ldpc_peg(n, k, var_degree, C.c_uint64(int(seed)), C.c_void_p(start.ctypes.data),
                       C.c_void_p(vars_.ctypes.data))
    if st != 0:
        raise ComrsError(st, L.cb_ldpc_last_error(None).decode())
    return [vars_[start[r]:start[r + 1]].tolist() for r in range(m)]


class Ldpc:
    """A sparse LDPC code of `n` variables and the checks `rows` on a GPU.

    ``encoder`` is ``"sums"`` (from_rows: the GF(2) elimination, on first use),
    ``"accumulate"`` (an IRA code, checked now) or None (a decoder only).
    """

    def __init__(self, n, rows, rule=DEFAULT_RULE, alpha=DEFAULT_ALPHA, layered=DEFAULT_LAYERED,
                 max_iterations=DEFAULT_MAX_ITERATIONS, precision="f64", device=0, encoder="sums"):
        from . import PRECISIONS, RULES, ComrsError, lib

        rule = _rule(rule)
        if encoder is not None and encoder not in ENCODERS:
            raise ComrsError(-1, f"encoder must be sums, accumulate or None, got {encoder!r}")
        if precision not in PRECISIONS:
            raise ComrsError(-1, f"precision must be f64 or f32, got {precision!r}")
        rows = [[int(v) for v in r] for r in rows]
        start = np.zeros(len(rows) + 1, np.int32)
        start[1:] = np.cumsum([len(r) for r in rows])
        vars_ = np.array([v for r in rows for v in r], np.int32)
        self._lib = lib()
        self._n, self.m, self._rows = int(n), len(rows), rows
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.rule, self.alpha, self.layered, self.max_iterations = rule, alpha, bool(layered), max_iterations
        h = C.c_void_p()
        st = self._lib.cb_ldpc_create(self._n, self.m, C.c_void_p(start.ctypes.data),
                                      C.c_void_p(vars_.ctypes.data if vars_.size else 0), RULES[rule],
                                      1.0 if rule == "min_sum" else float(alpha), int(bool(layered)),
                                      int(max_iterations), PRECISIONS[precision], device, C.byref(h))
        if st != 0:
            raise ComrsError(st, self._lib.cb_ldpc_last_error(None).decode())
        self._h = h
        self._encoder = encoder
        self._info = None
        if encoder == "accumulate":
            self._systematic()

    # ------------------------------------------------------------------ constructors
    @classmethod
    def peg(cls, n, k, *, var_degree=DEFAULT_VAR_DEGREE, seed=DEFAULT_PEG_SEED, **kw):
        """``LdpcCode.peg(n, k, var_degree=3, seed=1)``: progressive edge growth.

        >>> import importlib
        >>> cb = importlib.import_module("com-rs_gb300")
        >>> code = cb.Ldpc.peg(96, 48)
        >>> code.n, code.k, code.girth() >= 6
        (96, 48, True)
        """
        return cls(n, peg_rows(n, k, var_degree, seed), **kw)

    @classmethod
    def accumulate(cls, n, rows, **kw):
        """``LdpcCode::accumulate``: an IRA code (dual-diagonal parity part), encoded by
        accumulating its checks."""
        return cls(n, rows, encoder="accumulate", **kw)

    @classmethod
    def from_alist(cls, text, **kw):
        n, rows = parse_alist(text)
        return cls(n, rows, **kw)

    @classmethod
    def from_alist_file(cls, path, **kw):
        with open(path) as f:
            return cls.from_alist(f.read(), **kw)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cb_ldpc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __repr__(self):
        k = self._info.size if self._info is not None else "?"
        return f"LdpcCode(n={self._n}, k={k})"

    def _check(self, st):
        if st != 0:
            from . import ComrsError

            raise ComrsError(st, self._lib.cb_ldpc_last_error(self._h).decode())

    # ------------------------------------------------------------------ the code
    @property
    def n(self):
        """Coded bits per block."""
        return self._n

    @property
    def rows(self):
        """The rows of the parity-check matrix (the positions of their ones)."""
        return [list(r) for r in self._rows]

    def _systematic(self):
        if self._info is None:
            from . import ComrsError

            if self._encoder is None:
                raise ComrsError(-1, "the code was built without an encoder")
            k = C.c_int32()
            info = np.zeros(self._n, np.int32)
            self._check(self._lib.cb_ldpc_set_encoder(self._h, ENCODERS[self._encoder], C.byref(k),
                                                      C.c_void_p(info.ctypes.data)))
            self._info = info[:k.value].copy()
        return self._info

    @property
    def k(self):
        """Information bits per block (n - rank H)."""
        return int(self._systematic().size)

    @property
    def rate(self):
        """Code rate k / n."""
        return self.k / self._n

    def info_positions(self):
        """The positions of the information bits in the codeword, in their order."""
        return self._systematic().copy()

    def girth(self):
        """The length of the shortest cycle of the Tanner graph (0 without cycle)."""
        g = C.c_int32()
        self._check(self._lib.cb_ldpc_girth(self._h, C.byref(g)))
        return int(g.value)

    def to_alist(self):
        """The parity-check matrix in the alist format, lists padded with zeros
        (``LdpcCode::to_alist``, ldpc.rs:372-395)."""
        cols = [[] for _ in range(self._n)]
        for r, row in enumerate(self._rows):
            for v in row:
                cols[v].append(r)
        max_col = max((len(c) for c in cols), default=0)
        max_row = max((len(r) for r in self._rows), default=0)

        def line(values):
            return " ".join(str(v) for v in values) + "\n"

        def padded(lst, width):
            return line([v + 1 for v in lst] + [0] * (width - len(lst)))

        out = [f"{self._n} {self.m}\n{max_col} {max_row}\n", line(len(c) for c in cols),
               line(len(r) for r in self._rows)]
        out += [padded(c, max_col) for c in cols]
        out += [padded(r, max_row) for r in self._rows]
        return "".join(out)

    # ------------------------------------------------------------------ the decoder
    def set_decoder(self, rule=DEFAULT_RULE, *, alpha=DEFAULT_ALPHA, layered=DEFAULT_LAYERED,
                    max_iterations=DEFAULT_MAX_ITERATIONS):
        """Choose the decoder (``LdpcCode.set_decoder``): the rule, its scale or offset,
        the schedule and the iterations at most."""
        from . import RULES

        rule = _rule(rule)
        self._check(self._lib.cb_ldpc_set_decoder(self._h, RULES[rule], 1.0 if rule == "min_sum" else float(alpha),
                                                  int(bool(layered)), int(max_iterations)))
        self.rule, self.alpha, self.layered, self.max_iterations = rule, alpha, bool(layered), max_iterations

    def info(self):
        """n, m, edges, largest row and column degrees, levels, largest level, layered."""
        out = np.zeros(8, np.int64)
        self._check(self._lib.cb_ldpc_info(self._h, C.c_void_p(out.ctypes.data)))
        keys = ("n", "m", "edges", "max_row_degree", "max_col_degree", "levels", "max_level_rows", "layered")
        return dict(zip(keys, (int(x) for x in out)))

    def levels(self):
        """The layered schedule: (level_start, level_rows)."""
        inf = self.info()
        ls = np.zeros(inf["levels"] + 1, np.int32)
        lr = np.zeros(self.m, np.int32)
        self._check(self._lib.cb_ldpc_levels(self._h, C.c_void_p(ls.ctypes.data), C.c_void_p(lr.ctypes.data)))
        return ls, lr

    @staticmethod
    def _blocks(x, width, what):
        if x.ndim == 1 and x.size % width:
            raise ValueError(f"{what}: {x.size} values is not a multiple of {width}")
        if x.ndim == 2 and x.shape[1] != width:
            raise ValueError(f"{what}: rows of {x.shape[1]} values, expected {width}")
        if x.ndim not in (1, 2):
            raise ValueError(f"{what}: a 1-D or 2-D array is expected")
        return x.reshape(-1, width)

    def encode(self, bits):
        """Encode whole blocks: a multiple of `k` bits (1-D, the coded blocks one after
        the other) or rows of `k` bits (2-D, one coded block per row), on the GPU.

        >>> import importlib, numpy as np
        >>> cb = importlib.import_module("com-rs_gb300")
        >>> cb.Ldpc.peg(96, 48).encode(np.random.default_rng(1).integers(0, 2, 96)).size  # doctest: +SKIP
        192
        """
        k = self.k
        u = np.ascontiguousarray(bits, np.uint8)
        u2 = self._blocks(u, k, "bits")
        out = np.zeros((u2.shape[0], self._n), np.uint8)
        if u2.shape[0]:
            self._check(self._lib.cb_ldpc_encode(self._h, C.c_void_p(u2.ctypes.data), u2.shape[0],
                                                 C.c_void_p(out.ctypes.data)))
        return out.reshape(-1) if u.ndim == 1 else out

    def decode_llr(self, llr):
        """(posteriors, iterations) of one word (1-D) or of every row of a 2-D array."""
        x = np.ascontiguousarray(llr, self.dtype)
        single = x.ndim == 1
        if single and x.size != self._n:
            raise ValueError(f"llr: {x.size} values, expected {self._n}")
        x = self._blocks(x, self._n, "llr")
        post = np.zeros_like(x)
        its = np.zeros(x.shape[0], np.int32)
        self._check(self._lib.cb_ldpc_decode(self._h, C.c_void_p(x.ctypes.data), x.shape[0],
                                             C.c_void_p(post.ctypes.data), C.c_void_p(its.ctypes.data)))
        return (post[0], int(its[0])) if single else (post, its)

    def decode(self, llr):
        """Decode whole blocks of LLRs (positive for a 0): a multiple of `n` (1-D, the
        `k` decided information bits of every block one after the other) or rows of `n`
        (2-D, one row of `k` bits per block).

        >>> import importlib, numpy as np
        >>> cb = importlib.import_module("com-rs_gb300")
        >>> code = cb.Ldpc.peg(96, 48)
        >>> b = np.random.default_rng(1).integers(0, 2, 48).astype(np.uint8)
        >>> bool(np.array_equal(code.decode(2.0 - 4.0 * code.encode(b)), b))  # doctest: +SKIP
        True
        """
        x = np.ascontiguousarray(llr, self.dtype)
        x2 = self._blocks(x, self._n, "llr")
        post, _ = self.decode_llr(x2)
        bits = (post[:, self._systematic()] < 0).astype(np.uint8)
        return bits.reshape(-1) if x.ndim == 1 else bits

    def decode_block(self, llr, info_positions=None):
        """Hard decisions (1 for a negative posterior) at the information positions (the
        code's own unless given) of one word or of every row."""
        post, _ = self.decode_llr(llr)
        pos = self._systematic() if info_positions is None else np.asarray(info_positions)
        return (post[..., pos] < 0).astype(np.uint8)
