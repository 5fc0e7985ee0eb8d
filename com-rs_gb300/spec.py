"""com-spec specifications whose link is the BICM chain over a PEG LDPC code, on the GPU.

* :class:`Link` -- the link ``fec_encode -> map -> awgn_ebn0 -> demap -> fec_decode``
  (crates/com-spec/src/link.rs:109-124) over a generic :class:`Ldpc`, run by
  ``cb_link_run_trials``: one trial is ``blocks`` codewords, drawn from
  ``stream(seed, name, condition, trial)``, with the counts of the metrics ``ber``,
  ``coded_ber`` and ``bler`` (crates/com-spec/src/metrics.rs:254-351).
* :func:`load_yaml` -- the YAML that specification files are written in: block mappings
  and sequences, flow collections, anchors and aliases, plain and quoted scalars,
  comments.  Other YAML (tags, multi-line strings, documents) raises ValueError.
* :func:`run_spec` -- the campaign of a specification (crates/com-spec/src/spec.rs,
  run.rs): its grid (lists, ``{from, to, step}``, ``{linspace: [a, b, n]}``, scalars;
  spec.rs:373-406), seed, batch, the stopping rule ``(min_errors and min_trials) or
  max_trials`` (spec.rs:118-150) and the ``skip_below`` callback
  (crates/com-sim/src/callbacks.rs:168-203), with the conditions, batches and streams
  of com-sim's Runner.  Only the link above is built on the GPU; another link raises.
"""

import ctypes as C
import os
import re
import time

import numpy as np

from .campaign import ConditionResult, ErrorRate, Grid, Mean, Stop

LINK_DTYPE = np.dtype([("raw_bit_errors", "<u4"), ("coded_bit_errors", "<u4"), ("block_errors", "<u4"),
                       ("iterations", "<u4")])


class Link:
    """The BICM link of a specification over `code` (an f64 :class:`Ldpc` with the
    from_rows encoder): `blocks` codewords per trial, the random interleaver of
    `interleaver_seed` when `interleave` is set, Gray `modulation`-QAM, the exact (or
    max-log) demapper, and the code's decoder."""

    def __init__(self, code, blocks=1, modulation=4, interleave=False, interleaver_seed=0, demap="exact"):
        from . import ComrsError

        if demap not in ("exact", "max_log"):
            raise ComrsError(-1, f"demap must be exact or max_log, got {demap!r}")
        code.k  # the from_rows encoder, set on first use
        self.code, self._lib = code, code._lib
        h = C.c_void_p()
        st = self._lib.cb_link_create(code._h, int(blocks), int(modulation), int(bool(interleave)),
                                      C.c_uint64(int(interleaver_seed)), int(demap == "exact"), C.byref(h))
        if st != 0:
            raise ComrsError(st, self._lib.cb_link_last_error(None).decode())
        self._h = h
        inf = np.zeros(8, np.int64)
        self._check(self._lib.cb_link_info(self._h, C.c_void_p(inf.ctypes.data)))
        (self.k, self.n, self.blocks, self.modulation, self.sent_bits, self.payload_bits, self.padding,
         _) = (int(x) for x in inf)

    def _check(self, st):
        if st != 0:
            from . import ComrsError

            raise ComrsError(st, self._lib.cb_link_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cb_link_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def interleaver(self):
        """The permutation of the interleaver: stream bit t is coded bit perm[t]."""
        perm = np.zeros(self.n * self.blocks, np.int32)
        self._check(self._lib.cb_link_interleaver(self._h, C.c_void_p(perm.ctypes.data)))
        return perm

    def run_trials(self, seed, name, condition, first_trial, n_trials, ebn0_db):
        """The records (LINK_DTYPE) of trials [first_trial, first_trial + n_trials)."""
        from . import fnv1a64

        out = np.zeros(n_trials, LINK_DTYPE)
        if n_trials:
            self._check(self._lib.cb_link_run_trials(self._h, seed, fnv1a64(name), condition, first_trial, n_trials,
                                                     float(ebn0_db), C.c_void_p(out.ctypes.data)))
        return out

    def generate(self, seed, name, condition, first_trial, n_trials, ebn0_db):
        """(decoder LLRs [n_trials][n blocks], payload bits [n_trials][k blocks], uncoded
        bit errors [n_trials]) of the same trials."""
        from . import fnv1a64

        llr = np.zeros((n_trials, self.n * self.blocks))
        pay = np.zeros((n_trials, self.k * self.blocks), np.uint8)
        raw = np.zeros(n_trials, np.uint32)
        if n_trials:
            self._check(self._lib.cb_link_generate(self._h, seed, fnv1a64(name), condition, first_trial, n_trials,
                                                   float(ebn0_db), C.c_void_p(llr.ctypes.data),
                                                   C.c_void_p(pay.ctypes.data), C.c_void_p(raw.ctypes.data)))
        return llr, pay, raw


# ---------------------------------------------------------------------------- YAML

_FLOAT = re.compile(r"^[-+]?(\d+\.\d*|\.\d+|\d+)([eE][-+]?\d+)?$")
_INT = re.compile(r"^[-+]?\d+$")


def _scalar(tok):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"":
        if len(t) < 2 or t[-1] != t[0]:
            raise ValueError(f"yaml: unterminated string {t!r}")
        body = t[1:-1]
        return body.replace("''", "'") if t[0] == "'" else bytes(body, "utf-8").decode("unicode_escape")
    if t in ("null", "Null", "NULL", "~"):
        return None
    if t in ("true", "True", "TRUE"):
        return True
    if t in ("false", "False", "FALSE"):
        return False
    if _INT.match(t):
        return int(t)
    if _FLOAT.match(t):
        return float(t)
    if t in (".inf", "+.inf"):
        return float("inf")
    if t == "-.inf":
        return float("-inf")
    if t[0] in "!|>%@`":
        raise ValueError(f"yaml: {t!r} is not in the subset of YAML read here")
    return t


def _strip_comment(line):
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i].rstrip()
    return line.rstrip()


class _Flow:
    """A flow value ({...}, [...], an alias, an anchored value or a plain scalar)."""

    def __init__(self, text, anchors):
        self.s, self.i, self.anchors = text, 0, anchors

    def ws(self):
        while self.i < len(self.s) and self.s[self.i] in " \t\n":
            self.i += 1

    def value(self, stops):
        self.ws()
        anchor = None
        if self.s.startswith("&", self.i):
            m = re.compile(r"&([^\s,\[\]{}]+)").match(self.s, self.i)
            anchor, self.i = m.group(1), m.end()
            self.ws()
        if self.s.startswith("*", self.i):
            m = re.compile(r"\*([^\s,\[\]{}]+)").match(self.s, self.i)
            self.i = m.end()
            if m.group(1) not in self.anchors:
                raise ValueError(f"yaml: unknown alias *{m.group(1)}")
            v = self.anchors[m.group(1)]
        elif self.s.startswith("{", self.i):
            v = self.mapping()
        elif self.s.startswith("[", self.i):
            v = self.sequence()
        else:
            v = _scalar(self.token(stops))
        if anchor:
            self.anchors[anchor] = v
        return v

    def token(self, stops):
        start, q = self.i, None
        while self.i < len(self.s):
            ch = self.s[self.i]
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"" and self.i == start:
                q = ch
            elif ch in stops:
                break
            self.i += 1
        return self.s[start:self.i]

    def mapping(self):
        self.i += 1
        out = {}
        while True:
            self.ws()
            if self.s.startswith("}", self.i):
                self.i += 1
                return out
            key = _scalar(self.token(":,}"))
            self.ws()
            if self.s.startswith(":", self.i):
                self.i += 1
                out[key] = self.value(",}")
            else:
                out[key] = None
            self.ws()
            if self.s.startswith(",", self.i):
                self.i += 1
            elif not self.s.startswith("}", self.i):
                raise ValueError(f"yaml: expected , or }} in {self.s!r}")

    def sequence(self):
        self.i += 1
        out = []
        while True:
            self.ws()
            if self.s.startswith("]", self.i):
                self.i += 1
                return out
            out.append(self.value(",]"))
            self.ws()
            if self.s.startswith(",", self.i):
                self.i += 1
            elif not self.s.startswith("]", self.i):
                raise ValueError(f"yaml: expected , or ] in {self.s!r}")


def _balanced(text):
    depth, q = 0, None
    for ch in text:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch in "[{":
            depth += 1
        elif ch in "]}":
            depth -= 1
    return depth <= 0


class _Block:
    def __init__(self, text):
        self.lines = []
        for raw in text.splitlines():
            if raw.strip() in ("---", "..."):
                continue
            line = _strip_comment(raw)
            if line.strip():
                if "\t" in line[:len(line) - len(line.lstrip())]:
                    raise ValueError("yaml: tabs in the indentation")
                self.lines.append([len(line) - len(line.lstrip()), line.strip()])
        self.i, self.anchors = 0, {}

    def inline(self, rest):
        # a flow value may continue on the next lines until its brackets close
        while not _balanced(rest) and self.i < len(self.lines):
            rest += " " + self.lines[self.i][1]
            self.i += 1
        f = _Flow(rest, self.anchors)
        v = f.value("")
        f.ws()
        if f.i != len(f.s):
            raise ValueError(f"yaml: cannot read {rest!r}")
        return v

    def value_after(self, indent, rest):
        m = re.fullmatch(r"&([^\s]+)", rest)
        if rest and not m:
            return self.inline(rest)
        v = None
        if self.i < len(self.lines):
            ind, content = self.lines[self.i]
            if ind > indent or (ind == indent and content.startswith("-")):
                v = self.block(ind)
        if m:
            self.anchors[m.group(1)] = v
        return v

    def block(self, indent):
        content = self.lines[self.i][1]
        if content == "-" or content.startswith("- "):
            return self.sequence(indent)
        return self.mapping(indent)

    def mapping(self, indent):
        out = {}
        while self.i < len(self.lines):
            ind, content = self.lines[self.i]
            if ind < indent or (ind == indent and content.startswith("-")):
                break
            if ind > indent:
                raise ValueError(f"yaml: unexpected indentation at {content!r}")
            m = re.match(r"^('[^']*'|\"[^\"]*\"|[^:]+?)\s*:(\s+|$)(.*)$", content)
            if not m:
                raise ValueError(f"yaml: expected key: value, got {content!r}")
            self.i += 1
            out[_scalar(m.group(1))] = self.value_after(indent, m.group(3).strip())
        return out

    def sequence(self, indent):
        out = []
        while self.i < len(self.lines):
            ind, content = self.lines[self.i]
            if ind != indent or not (content == "-" or content.startswith("- ")):
                break
            item = content[1:].strip()
            if not item:
                self.i += 1
                out.append(self.value_after(indent, ""))
            elif item == "-" or item.startswith("- "):
                # "- - x": a sequence whose items sit two columns in
                self.lines[self.i] = [indent + 2, item]
                out.append(self.sequence(indent + 2))
            elif re.match(r"^[^\s{\[\"'&*][^:{}\[\]]*:(\s|$)", item):
                # "- key: value": a mapping whose keys sit two columns in
                self.lines[self.i] = [indent + 2, item]
                out.append(self.mapping(indent + 2))
            else:
                self.i += 1
                out.append(self.inline(item))
        return out


def load_yaml(text):
    """The value of a YAML text in the subset the specification files use."""
    b = _Block(text)
    if not b.lines:
        return None
    v = b.block(b.lines[0][0])
    if b.i != len(b.lines):
        raise ValueError(f"yaml: cannot read {b.lines[b.i][1]!r}")
    return v


# ---------------------------------------------------------------------------- specs

_QAM = {"qpsk": 4, "4qam": 4, "16qam": 16, "64qam": 64, "256qam": 256}


def _modulation(name):
    # Constellation::from_name (crates/com-mapping/src/constellation.rs:254-270), QAM only
    key = str(name).lower().replace("-", "").replace("_", "").replace(" ", "")
    if key not in _QAM:
        raise ValueError(f"map: the GPU link has the Gray QAM of order 4, 16, 64 or 256, got {name!r}")
    return _QAM[key]


def _axis(name, v):
    # grid_axis (crates/com-spec/src/spec.rs:373-406)
    if isinstance(v, list):
        return v
    if isinstance(v, dict):
        if "linspace" in v:
            a, b, n = v["linspace"]
            n = int(n)
            return [a if n == 1 else a + (b - a) * i / (n - 1) for i in range(n)]
        a, b, st = v.get("from"), v.get("to"), v.get("step")
        if None in (a, b, st) or st == 0 or (b - a) / st < 0:
            raise ValueError(f"grid {name!r}: an axis is a list, {{from, to, step}} or {{linspace: [start, stop, count]}}")
        n = int(np.floor((b - a) / st + 1e-9)) + 1
        ints = all(isinstance(x, int) and not isinstance(x, bool) for x in (a, b, st))
        return [int(a + st * i) if ints else float(a + st * i) for i in range(n)]
    return [v]


def _stop(q):
    # StopSpec::rule (spec.rs:118-150): (all targets and min_trials) or the caps
    unknown = set(q) - {"max_trials", "min_trials", "min_errors", "precision", "max_time_s"}
    if unknown or q.get("precision") or q.get("max_time_s") is not None:
        raise ValueError(f"stop: the GPU runner reads max_trials, min_trials and min_errors, got {sorted(q)}")
    targets = [Stop.min_errors(m, int(k)) for m, k in (q.get("min_errors") or {}).items()]
    caps = [Stop.max_trials(int(q["max_trials"]))] if q.get("max_trials") is not None else []
    if not targets and not caps:
        caps.append(Stop.max_trials(max(int(q.get("min_trials") or 100), 1)))
    any_ = []
    if targets:
        if q.get("min_trials") is not None:
            targets.append(Stop.min_trials(int(q["min_trials"])))
        any_.append(targets[0] if len(targets) == 1 else Stop("all", rules=targets))
    any_ += caps
    return any_[0] if len(any_) == 1 else Stop("any", rules=any_)


def _block(b):
    if isinstance(b, str):
        return b, {}
    if isinstance(b, dict) and "type" in b:
        return b["type"], {k: v for k, v in b.items() if k != "type"}
    raise ValueError(f"link: a block is a name or a mapping with a type, got {b!r}")


def _link_settings(link):
    """The settings of the one link the GPU runs, from the blocks of a specification."""
    kinds = [_block(b) for b in link]
    if [k for k, _ in kinds] != ["fec_encode", "map", "awgn_ebn0", "demap", "fec_decode"]:
        raise ValueError("link: the GPU runs fec_encode, map, awgn_ebn0, demap, fec_decode, got "
                         f"{[k for k, _ in kinds]}")
    enc, mp, awgn, dm, dec = (p for _, p in kinds)
    if awgn.get("ebn0_db") is None:
        raise ValueError("awgn_ebn0: ebn0_db is required")
    code, dcode = enc.get("code"), dec.get("code")
    for c in (code, dcode):
        if not isinstance(c, dict) or c.get("type") != "ldpc":
            raise ValueError(f"fec_encode/fec_decode: the GPU link takes an ldpc code, got {c!r}")
    construction = ("n", "k", "var_degree", "seed")
    if any(code.get(x) != dcode.get(x) for x in construction):
        raise ValueError("fec_encode and fec_decode must build the same code")
    if (bool(enc.get("interleave", False)), enc.get("seed", 0)) != (bool(dec.get("interleave", False)),
                                                                    dec.get("seed", 0)):
        raise ValueError("fec_encode and fec_decode must give the same interleaver")
    return {
        "n": int(code["n"]), "k": int(code["k"]), "var_degree": int(code.get("var_degree", 3)),
        "peg_seed": int(code.get("seed", 1)),
        "rule": dcode.get("rule", "sum_product"), "alpha": float(dcode.get("alpha", 0.8)),
        "layered": bool(dcode.get("layered", True)), "iterations": int(dcode.get("iterations", 50)),
        "blocks": int(enc.get("blocks", 1)), "interleave": bool(enc.get("interleave", False)),
        "interleaver_seed": int(enc.get("seed", 0)),
        "modulation": _modulation(mp.get("constellation", "QPSK")),
        "ebn0_db": awgn.get("ebn0_db"), "demap": "max_log" if dm.get("max_log", False) else "exact",
    }


def build_link(spec, device=0):
    """The :class:`Link` of a specification (its code built by progressive edge growth)."""
    from .ldpc import Ldpc

    s = _link_settings(spec["link"])
    code = Ldpc.peg(s["n"], s["k"], var_degree=s["var_degree"], seed=s["peg_seed"], rule=s["rule"], alpha=s["alpha"],
                    layered=s["layered"], max_iterations=s["iterations"], device=device)
    return Link(code, s["blocks"], s["modulation"], s["interleave"], s["interleaver_seed"], s["demap"]), s


def _value(v, cond):
    if isinstance(v, str) and v.startswith("$"):
        if v[1:] not in cond:
            raise ValueError(f"the variable {v} is not on the grid")
        return cond[v[1:]]
    return v


def _parse(spec):
    if isinstance(spec, str):
        spec = load_yaml(open(spec).read() if os.path.exists(spec) else spec)
    return spec


def run_spec(spec, device=0, on_batch=None, rank=0, world=1, all_reduce=None):
    """The campaign of a specification (a mapping, a YAML text or a file name): one
    ConditionResult per condition in grid order, with the ErrorRate of every reported
    metric (``ber``, ``coded_ber``, ``bler``) and the decoder's iterations per block;
    conditions that ``skip_below`` skips come back with status ``skipped``.

    Several processes (one GPU each) run one campaign together as :func:`run` does:
    process ``rank`` of ``world`` runs its contiguous share of every batch, and
    ``all_reduce`` (summing an int64 vector over the processes) merges the counts before
    the stop rule; the result equals the one-process campaign."""
    from . import fnv1a64  # noqa: F401  (the library must load before any work)

    spec = _parse(spec)
    link, s = build_link(spec, device)
    try:
        return run_spec_with(link, spec, on_batch, rank, world, all_reduce)
    finally:
        link.close()


def run_spec_with(link, spec, on_batch=None, rank=0, world=1, all_reduce=None):
    """The campaign of `spec` on `link`: anything with run_trials(seed, name, condition,
    first_trial, n_trials, ebn0_db) returning LINK_DTYPE records and the attributes
    sent_bits, payload_bits and blocks (:class:`Link`, or a stand-in computing the same
    trials elsewhere)."""
    spec = _parse(spec)
    if world > 1 and all_reduce is None:
        raise ValueError("a multi-process campaign needs all_reduce")
    s = _link_settings(spec["link"])
    name, seed, batch = spec["name"], int(spec.get("seed", 0)), max(1, int(spec.get("batch", 32)))
    grid = Grid()
    for k, v in (spec.get("grid") or {}).items():
        grid.axis(k, _axis(k, v))
    metrics = spec.get("metrics") or {}
    report = [m.lower() for m in (metrics.get("report") or ["ber", "coded_ber", "bler"])]
    if set(report) - {"ber", "coded_ber", "bler"}:
        raise ValueError(f"metrics: the GPU link reports ber, coded_ber and bler, got {report}")
    stop = _stop(spec.get("stop") or {})
    if not stop.is_bounded():
        raise ValueError("the stopping rule can run forever: add max_trials")
    skip = ((spec.get("callbacks") or {}).get("skip_below"))
    done, results = [], []
    for index, cond in enumerate(grid.conditions()):
        others = sorted((k, v) for k, v in cond.items() if not skip or k != skip["along"])
        if skip and others in done:
            results.append(ConditionResult(index, cond, 0, 0.0, {}, "skipped"))
            continue
        ebn0 = float(_value(s["ebn0_db"], cond))
        t0 = time.perf_counter()
        rec = {m: ErrorRate() for m in report}
        its = Mean()
        trials, limit = 0, stop.trial_limit()
        while True:
            end = trials + batch if limit is None else max(min(trials + batch, limit), trials + 1)
            n = end - trials
            lo, hi = trials + n * rank // world, trials + n * (rank + 1) // world
            counts = np.zeros(4, np.int64)
            if hi > lo:
                r = link.run_trials(seed, name, index, lo, hi - lo, ebn0)
                counts[:] = (r["raw_bit_errors"].sum(dtype="u8"), r["coded_bit_errors"].sum(dtype="u8"),
                             r["block_errors"].sum(dtype="u8"), r["iterations"].sum(dtype="u8"))
            if world > 1:
                counts = all_reduce(counts)
            if "ber" in rec:
                rec["ber"].add(int(counts[0]), link.sent_bits * n)
            if "coded_ber" in rec:
                rec["coded_ber"].add(int(counts[1]), link.payload_bits * n)
            if "bler" in rec:
                rec["bler"].add(int(counts[2]), link.blocks * n)
            its.add_many(n * link.blocks, int(counts[3]))
            trials = end
            if on_batch:
                on_batch(index, trials, rec)
            if stop.is_met(trials, rec):
                break
        rec["iterations"] = its
        results.append(ConditionResult(index, cond, trials, time.perf_counter() - t0, rec))
        if skip:
            e = rec.get(skip["metric"].lower())
            if trials > 0 and e is not None and e.rate() < float(skip["threshold"]) and others not in done:
                done.append(others)
    return results
