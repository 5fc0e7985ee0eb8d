"""The graph-specialised f32 layered decoder (csrc/layered_nr.cuh).

The library builds it once per base graph (Z and the shifts from the launch parameters)
and, per code, again at run time with Z and every shift as constants.  Both builds must
give the f32 oracle's decisions, iteration counts and a posteriori LLRs bit for bit; the
base graph's build is forced in a child process by COMRS_NO_JIT=1.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CODES = [
    dict(k=8448, e=25344, bg=1, z=384, m=16, eb=2.7),                 # benchmark config 2
    dict(k=520, e=1040, bg=2, z=52, m=4, eb=1.5),                     # benchmark config 1
    dict(k=100, e=300, m=4, eb=1.0),                                  # fillers: K' < K
    dict(k=60, e=1000, rv=1, qm=2, m=4, eb=-2.0),                     # repeated bits (E > N_cb)
    dict(k=500, e=1200, rv=2, qm=4, m=16, eb=2.0),                    # positions map
    dict(k=20, e=60, bg=2, z=2, m=4, eb=2.0),                         # the smallest lifting
    dict(k=2000, e=4200, bg=1, z=96, m=16, eb=2.5, rule="offset_min_sum", alpha=0.15),
]

CHILD = r"""
import importlib, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
cb = importlib.import_module("com-rs_gb300")
d = np.load(sys.argv[2], allow_pickle=True)
s = d["spec"].item()
g = cb.NrLdpc(s["k"], s["e"], base_graph=s.get("bg"), lifting_size=s.get("z"), rv=s.get("rv", 0), qm=s.get("qm", 1),
              precision="f32", rule=s.get("rule", "normalized_min_sum"), alpha=s.get("alpha", 0.75))
bits, app, it = g.decode_full(d["llr"])
np.savez(sys.argv[3], bits=bits, app=app, it=it, decoder=g.decoder)
"""


def build(cb, spec):
    return cb.NrLdpc(spec["k"], spec["e"], base_graph=spec.get("bg"), lifting_size=spec.get("z"), rv=spec.get("rv", 0),
                     qm=spec.get("qm", 1), precision="f32", rule=spec.get("rule", "normalized_min_sum"),
                     alpha=spec.get("alpha", 0.75))


def frames(O, spec, n):
    ref = O.Code(spec["k"], spec["e"], bg=spec.get("bg", 0), z=spec.get("z", 0), rv=spec.get("rv", 0),
                 qm=spec.get("qm", 1))
    rule = O.RULE_OMS if spec.get("rule") == "offset_min_sum" else O.RULE_NMS
    ref.set_decoder(rule, spec.get("alpha", 0.75), True, 20)
    llr = np.zeros((n, spec["e"]))
    h = O.fnv1a64("nr_kernel")
    for f in range(n):
        _, llr[f], _ = ref.trial(spec["m"], 11, h, 0, f, spec["eb"])
    return ref, llr.astype(np.float32)


def test_the_benchmark_code_runs_its_own_build(cb):
    g = build(cb, CODES[0])
    assert g.decoder == "not yet on a device"
    g.decode(np.zeros((1, CODES[0]["e"]), np.float32))
    assert g.decoder == "layered min-sum compiled for this lifting"
    f64 = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f64")
    f64.decode(np.zeros((1, 1040)))
    assert f64.decoder == "generic layered"


@pytest.mark.parametrize("spec", CODES, ids=lambda s: f"k{s['k']}_e{s['e']}_{s.get('rule', 'nms')}")
def test_both_builds_equal_the_f32_oracle(cb, O, spec, tmp_path):
    n = 6 if spec["k"] > 4000 else 24
    ref, llr = frames(O, spec, n)
    g = build(cb, spec)
    bits, app, it = g.decode_full(llr)
    assert g.decoder == "layered min-sum compiled for this lifting"
    for f in range(n):
        rb, rit, rapp, _ = ref.decode(llr[f], "f32", want_app=True)
        assert np.array_equal(bits[f], rb) and it[f] == rit, f
        assert np.array_equal(app[f].view(np.uint32), rapp.view(np.uint32)), f
    # the base graph's build, in a child process without the run-time compiler
    src, out = tmp_path / "in.npz", tmp_path / "out.npz"
    np.savez(src, llr=llr, spec=np.array(spec, dtype=object))
    env = dict(os.environ, COMRS_NO_JIT="1")
    subprocess.run([sys.executable, "-c", CHILD, ROOT, str(src), str(out)], env=env, check=True, timeout=600)
    other = np.load(out)
    assert str(other["decoder"]) == "base-graph layered min-sum"
    assert np.array_equal(other["bits"], bits) and np.array_equal(other["it"], it)
    assert np.array_equal(other["app"].view(np.uint32), app.view(np.uint32))
