"""Mixed batches: every record of the persistent mixed kernel equals the single-code
path (cb_run_frames of the item's own code on the same stream position), whatever the
rows per thread the autotuner picks, and the oracle's f32 decoder on the LLRs the batch
generates."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAME = "mixtest"


def single_code_records(cb, items, epoch, n):
    codes, out = {}, []
    for it in items:
        key = (int(it["base_graph"]), int(it["lifting_size"]), int(it["k_info"]), int(it["e"]))
        g = codes.get(key)
        if g is None:
            g = codes[key] = cb.NrLdpc(key[2], key[3], base_graph=key[0], lifting_size=key[1], precision="f32",
                                       max_iterations=25)
        out.append(g.run_frames(7, NAME, int(it["condition"]), int(it["frame"]) + epoch * n, 1, float(it["ebn0_db"]),
                                int(it["modulation_order"]))[0])
    return np.array(out, dtype=cb.FRAME_DTYPE)


def test_mixed_batch_equals_the_single_code_path(cb):
    items = cb.draw_mixed_batch(n=300, seed=5)
    mix = cb.MixBatch(items, seed=7, name=NAME, max_iterations=25)
    classes = mix.classes()
    assert sorted(c["z"] for c in classes) == sorted(set(int(z) for z in items["lifting_size"]))
    assert sum(c["count"] for c in classes) == len(items)
    for epoch in (0, 1):
        got = mix.run(epoch)
        want = single_code_records(cb, items, epoch, len(items))
        assert np.array_equal(got, want), epoch
    # some frames decode, some fail, early exits differ per codeword
    assert 0 < got["frame_error"].sum() < len(items) and len(set(got["iterations"])) > 3


def test_mixed_batch_decodes_as_the_oracle(cb, O):
    # The oracle anchor: every item's LLRs, as the batch's generator writes them, decoded
    # by the oracle's f32 layered min-sum (the same algorithm in f32, 25 iterations): the
    # same iteration count and the same bit errors against the item's information bits,
    # which are the oracle's own draws of that stream position.
    items = cb.draw_mixed_batch(n=300, seed=5)
    mix = cb.MixBatch(items, seed=7, name=NAME, max_iterations=25)
    for epoch in (0, 1):
        got = mix.run(epoch)
        llrs, infos = mix.frames(epoch)
        codes = {}
        for i, it in enumerate(items):
            key = (int(it["base_graph"]), int(it["lifting_size"]), int(it["k_info"]), int(it["e"]))
            ref = codes.get(key)
            if ref is None:
                ref = codes[key] = O.Code(key[2], key[3], bg=key[0], z=key[1]).set_decoder(O.RULE_NMS, 0.75, True, 25)
            frame = int(it["frame"]) + epoch * len(items)
            rinfo, _, _ = ref.trial(int(it["modulation_order"]), 7, O.fnv1a64(NAME), int(it["condition"]), frame,
                                    float(it["ebn0_db"]))
            assert np.array_equal(infos[i], rinfo), i
            bits, iters, _, _ = ref.decode(llrs[i], "f32")
            assert iters == got["iterations"][i], (i, iters, got["iterations"][i])
            assert int(np.sum(bits != rinfo)) == got["bit_errors"][i], i
            assert bool(got["frame_error"][i]) == bool(np.any(bits != rinfo)), i


def test_rows_per_thread_do_not_change_the_records(cb):
    items = cb.draw_mixed_batch(n=200, seed=9, zs=(64, 128, 384))
    mix = cb.MixBatch(items, seed=7, name=NAME, max_iterations=25)
    base = mix.run(0)
    for k, c in enumerate(mix.classes()):
        for rho in (2,):
            try:
                mix.set_rows_per_thread(k, rho)
            except cb.ComrsError:
                continue
            assert np.array_equal(mix.run(0), base), (c["z"], rho)
        mix.set_rows_per_thread(k, 1)


def test_autotuner_picks_a_layout_per_class(cb, tmp_path, monkeypatch):
    monkeypatch.setenv("COMRS_GB300_CACHE", str(tmp_path))
    items = cb.draw_mixed_batch(n=512, seed=3, zs=(32, 128))
    mix = cb.MixBatch(items, seed=7, name=NAME, max_iterations=25)
    base = mix.run(0)
    chosen = cb.autotune(mix, reps=1)
    assert set(chosen) == {32, 128}
    for z, (rho, times) in chosen.items():
        assert rho in times and times[rho] == min(times.values())
    assert np.array_equal(mix.run(0), base)
    again = cb.autotune(mix, reps=1)  # from the cache
    assert {z: r for z, (r, _) in again.items()} == {z: r for z, (r, _) in chosen.items()}
