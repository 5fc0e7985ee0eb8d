"""The LDPC codes of DVB-S2 (ETSI EN 302 307-1) for the generic GPU decoder.

Follows ``crates/com-systems/src/dvbs2/fec.rs``: the (k_bch, k_ldpc, t) of Tables 5a and
5b with their address tables (``params``, fec.rs:173-210), and the rows of H
(``ldpc_rows``, fec.rs:213-235): information bit l of group j, with the group's
addresses x, sits in the checks (x + l q) mod (n - k), q = (n - k) / 360; check r then
closes on the parity bits k + r - 1 (r > 0) and k + r, the dual-diagonal accumulator.
The code is the IRA code of ``LdpcCode::accumulate`` and its decoder defaults to the
sum-product rule, as ``Dvbs2Fec::new`` sets them (fec.rs:262-264).

Only the LDPC part is here (the outer BCH code is not on the GPU path).
"""

from .dvbs2_tables import TABLES

FRAMES = {"normal": 64800, "short": 16200}

# rate -> (k_bch, k_ldpc, t) per frame (Tables 5a and 5b)
PARAMS = {
    "normal": {"1/4": (16008, 16200, 12), "1/3": (21408, 21600, 12), "2/5": (25728, 25920, 12),
               "1/2": (32208, 32400, 12), "3/5": (38688, 38880, 12), "2/3": (43040, 43200, 10),
               "3/4": (48408, 48600, 12), "4/5": (51648, 51840, 12), "5/6": (53840, 54000, 10),
               "8/9": (57472, 57600, 8), "9/10": (58192, 58320, 8)},
    "short": {"1/4": (3072, 3240, 12), "1/3": (5232, 5400, 12), "2/5": (6312, 6480, 12),
              "1/2": (7032, 7200, 12), "3/5": (9552, 9720, 12), "2/3": (10632, 10800, 12),
              "3/4": (11712, 11880, 12), "4/5": (12432, 12600, 12), "5/6": (13152, 13320, 12),
              "8/9": (14232, 14400, 12)},
}


def params(frame, rate):
    """(n, k_bch, k_ldpc, t, address groups) of a frame size and a rate."""
    frame = str(frame).lower()
    if frame in ("64800",):
        frame = "normal"
    if frame in ("16200",):
        frame = "short"
    if frame not in FRAMES:
        raise ValueError(f"frame must be normal (64800) or short (16200), got {frame!r}")
    if frame == "short" and rate == "9/10":
        raise ValueError("DVB-S2 has no short FECFRAME of rate 9/10")
    if rate not in PARAMS[frame]:
        raise ValueError(f"rate must be one of {sorted(PARAMS[frame])}, got {rate!r}")
    n = FRAMES[frame]
    k_bch, k_ldpc, t = PARAMS[frame][rate]
    return n, k_bch, k_ldpc, t, TABLES[f"N{n}_P{n - k_ldpc}"]


def ldpc_rows(frame, rate):
    """(n, k, rows of H) of the LDPC code."""
    n, _, k, _, groups = params(frame, rate)
    m = n - k
    q = m // 360
    rows = [[] for _ in range(m)]
    bit = 0
    for addresses in groups:
        for l in range(360):
            for x in addresses:
                rows[(x + l * q) % m].append(bit)
            bit += 1
    for r, row in enumerate(rows):
        if r > 0:
            row.append(k + r - 1)
        row.append(k + r)
    return n, k, rows


def Dvbs2Ldpc(frame, rate, rule="sum_product", **decoder):
    """The LDPC code of a DVB-S2 FECFRAME on the GPU (an :class:`Ldpc`), with the
    accumulate encoder of ``LdpcCode::accumulate`` as ``Dvbs2Fec::new`` builds it
    (fec.rs:262)."""
    from .ldpc import Ldpc

    n, k, rows = ldpc_rows(frame, rate)
    code = Ldpc.accumulate(n, rows, rule=rule, **decoder)
    assert code.k == k
    return code
