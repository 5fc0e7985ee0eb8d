"""Re-create the golden fixtures of this directory from the reference's own test data.

Run in a checkout where the com-rs sources are available (they are not needed to run the
tests):  ``python tests/golden/make_golden.py <com-rs root>``

Outputs (committed):
  * ``sionna_nr_ldpc.npz`` -- the 28 NR-LDPC (K', E) encodings of the reference's
    fixture ``tests/oracle/sionna_vectors.npz`` (keys ``ldpc.k{K}_n{E}.{u,c}``,
    Apache-2.0, provenance in ``tests/oracle/sionna_vectors.json`` of com-rs), stored
    with np.packbits along the last axis (shape kept in ``<key>.shape``);
  * the AFF3CT FER/BER curves of the LDPC decoders on com-rs's PEG matrices
    (``validation/aff3ct/`` of com-rs): ``ldpc_peg_n576_k288_layered_nms075_i20.json``
    (layered normalised min-sum 0.75, 20 iterations), ``..._flooding_oms015_i20.json``
    (flooding offset min-sum 0.15), ``..._flooding_spa_i50.json`` (flooding
    sum-product, 50 iterations) and ``ldpc_peg_n648_k540_layered_spa_i20.json``
    (layered sum-product), with their matrices ``peg_n576_k288.alist`` and
    ``peg_n648_k540.alist``, and ``ldpc_dvbs2_short_r1_2_layered_spa_i50.json`` (the
    DVB-S2 short rate-1/2 LDPC code, layered sum-product, 50 iterations).
"""

import json
import os
import shutil
import sys

import numpy as np


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "."
    here = os.path.dirname(os.path.abspath(__file__))
    src = np.load(os.path.join(root, "tests/oracle/sionna_vectors.npz"))
    out = {}
    for k in sorted(src.files):
        if not k.startswith("ldpc."):
            continue
        a = np.asarray(src[k], dtype=np.uint8)
        out[k] = np.packbits(a, axis=-1)
        out[k + ".shape"] = np.array(a.shape, dtype=np.int64)
    np.savez_compressed(os.path.join(here, "sionna_nr_ldpc.npz"), **out)
    prov = json.load(open(os.path.join(root, "tests/oracle/sionna_vectors.json")))
    json.dump({"source": "com-rs tests/oracle/sionna_vectors.npz", "upstream_commit": prov.get("commit"),
               "keys": sorted(k for k in out if not k.endswith(".shape"))},
              open(os.path.join(here, "sionna_nr_ldpc.json"), "w"), indent=1)
    for name in ("ldpc_peg_n576_k288_layered_nms075_i20", "ldpc_peg_n576_k288_flooding_oms015_i20",
                 "ldpc_peg_n576_k288_flooding_spa_i50", "ldpc_peg_n648_k540_layered_spa_i20",
                 "ldpc_dvbs2_short_r1_2_layered_spa_i50"):
        shutil.copy(os.path.join(root, "validation/aff3ct", name + ".json"), os.path.join(here, name + ".json"))
    for m in ("peg_n576_k288.alist", "peg_n648_k540.alist"):
        shutil.copy(os.path.join(root, "validation/aff3ct/matrices", m), os.path.join(here, m))


if __name__ == "__main__":
    main()
