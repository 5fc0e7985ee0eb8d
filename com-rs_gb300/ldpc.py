"""Generic sparse LDPC codes on the GPU: the reference's ``LdpcCode`` decoder for any
parity-check matrix (crates/com-fec/src/ldpc.rs).

* :func:`parse_alist` -- MacKay's ``alist`` format with the checks of the reference's
  parser (ldpc.rs:638-741): comments after ``#``, lists padded with zeros or not,
  degrees that reach their declared maxima, 1-based indices in range and not repeated,
  column and row lists that agree.  It returns ``(n, rows)``, rows in file order.
* :class:`Ldpc` -- a code of ``n`` variables and the given rows, decoded on the GPU by
  ``cb_ldpc_decode`` with the settings of ``LdpcDecoder`` (ldpc.rs:165-172): rule
  ``sum_product``, ``min_sum``, ``normalized_min_sum`` or ``offset_min_sum``
  (``CheckRule::from_name``, ldpc.rs:104-113), layered or flooding schedule, maximum
  iterations.  :meth:`Ldpc.decode_llr` returns the posteriors and the iterations used
  (``LdpcCode::decode_llr``, ldpc.rs:497-505); :meth:`Ldpc.decode_block` the hard
  decisions at the information positions the caller gives (``decode_block``,
  ldpc.rs:793-796).

There is no CPU decoder here: without the CUDA library the calls raise.
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


class Ldpc:
    """A sparse LDPC code of `n` variables and the checks `rows` on a GPU."""

    def __init__(self, n, rows, rule=DEFAULT_RULE, alpha=DEFAULT_ALPHA, layered=DEFAULT_LAYERED,
                 max_iterations=DEFAULT_MAX_ITERATIONS, precision="f64", device=0):
        from . import PRECISIONS, RULES, ComrsError, lib

        if rule not in RULES:
            raise ComrsError(-1, "rule must be sum_product, min_sum, normalized_min_sum or offset_min_sum, "
                                 f"got {rule!r}")
        if rule == "min_sum":
            alpha = 1.0
        rows = [list(r) for r in rows]
        start = np.zeros(len(rows) + 1, np.int32)
        start[1:] = np.cumsum([len(r) for r in rows])
        vars_ = np.array([v for r in rows for v in r], np.int32)
        self._lib = lib()
        self.n, self.m, self.rows = int(n), len(rows), rows
        self.dtype = np.float64 if precision == "f64" else np.float32
        self.rule, self.alpha, self.layered, self.max_iterations = rule, alpha, bool(layered), max_iterations
        h = C.c_void_p()
        st = self._lib.cb_ldpc_create(self.n, self.m, C.c_void_p(start.ctypes.data),
                                      C.c_void_p(vars_.ctypes.data if vars_.size else 0), RULES[rule], float(alpha),
                                      int(bool(layered)), int(max_iterations), PRECISIONS[precision], device,
                                      C.byref(h))
        if st != 0:
            raise ComrsError(st, self._lib.cb_ldpc_last_error(None).decode())
        self._h = h

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

    def _check(self, st):
        if st != 0:
            from . import ComrsError

            raise ComrsError(st, self._lib.cb_ldpc_last_error(self._h).decode())

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

    def decode_llr(self, llr):
        """(posteriors, iterations) of one word (1-D) or of every row of a 2-D array."""
        x = np.ascontiguousarray(llr, self.dtype)
        single = x.ndim == 1
        x = x.reshape(-1, self.n)
        post = np.zeros_like(x)
        its = np.zeros(x.shape[0], np.int32)
        self._check(self._lib.cb_ldpc_decode(self._h, C.c_void_p(x.ctypes.data), x.shape[0],
                                             C.c_void_p(post.ctypes.data), C.c_void_p(its.ctypes.data)))
        return (post[0], int(its[0])) if single else (post, its)

    def decode_block(self, llr, info_positions):
        """Hard decisions (1 for a negative posterior) at the information positions."""
        post, _ = self.decode_llr(llr)
        return (post[..., np.asarray(info_positions)] < 0).astype(np.uint8)
