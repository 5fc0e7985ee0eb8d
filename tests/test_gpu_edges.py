"""Zero frames, trials or words through every entry point that takes a count: each
returns CB_OK and leaves its outputs as they were (the reference's decoders and runners
take empty batches the same way)."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_zero_counts_are_no_ops(cb):
    import torch

    L = cb.lib()
    code = cb.NrLdpc(520, 1040, base_graph=2, lifting_size=52, precision="f32")
    net = cb.LearnedNms(code, 4, shared=True)
    peg = cb.Ldpc.peg(96, 48)
    link = cb.Link(peg, blocks=2, modulation=16, interleave=True, interleaver_seed=3, demap="max_log")
    host = np.full(1 << 16, 0x5A, np.uint8)
    dev = torch.full((1 << 16,), 0x5A, dtype=torch.uint8, device="cuda")
    hp, dp = C.c_void_p(host.ctypes.data), C.c_void_p(dev.data_ptr())
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    h = cb.fnv1a64("zero")
    calls = {
        "cb_encode": lambda: L.cb_encode(code._h, hp, 0, hp),
        "cb_decode": lambda: L.cb_decode(code._h, hp, 0, hp, hp, hp),
        "cb_decode_device": lambda: L.cb_decode_device(code._h, dp, 0, dp, dp, dp, s),
        "cb_run_frames": lambda: L.cb_run_frames(code._h, 4, 1, h, 0, 0, 0, 1.0, hp),
        "cb_run_frames_device": lambda: L.cb_run_frames_device(code._h, 4, 1, h, 0, 0, 0, 1.0, dp, s),
        "cb_generate_frames": lambda: L.cb_generate_frames(code._h, 4, 1, h, 0, 0, 0, 1.0, hp, hp),
        "cb_generate_frames_device": lambda: L.cb_generate_frames_device(code._h, 4, 1, h, 0, 0, 0, 1.0, dp, dp, s),
        "cb_nms_forward": lambda: L.cb_nms_forward(net._h, hp, 0, hp),
        "cb_nms_decode": lambda: L.cb_nms_decode(net._h, hp, 0, hp, hp),
        "cb_nms_decode_device": lambda: L.cb_nms_decode_device(net._h, dp, 0, dp, dp, s),
        "cb_nms_run_frames": lambda: L.cb_nms_run_frames(net._h, 4, 1, h, 0, 0, 0, 1.0, hp),
        "cb_ldpc_encode": lambda: L.cb_ldpc_encode(peg._h, hp, 0, hp),
        "cb_ldpc_encode_device": lambda: L.cb_ldpc_encode_device(peg._h, dp, 0, dp, s),
        "cb_ldpc_decode": lambda: L.cb_ldpc_decode(peg._h, hp, 0, hp, hp),
        "cb_ldpc_decode_device": lambda: L.cb_ldpc_decode_device(peg._h, dp, 0, dp, dp, s),
        "cb_link_run_trials": lambda: L.cb_link_run_trials(link._h, 1, h, 0, 0, 0, 3.0, hp),
        "cb_link_run_trials_device": lambda: L.cb_link_run_trials_device(link._h, 1, h, 0, 0, 0, 3.0, dp, s),
        "cb_link_generate": lambda: L.cb_link_generate(link._h, 1, h, 0, 0, 0, 3.0, hp, hp, hp),
    }
    failed = {name: st for name, st in ((name, call()) for name, call in calls.items()) if st != 0}
    torch.cuda.synchronize()
    assert not failed, failed
    assert (host == 0x5A).all()
    assert bool((dev == 0x5A).all())
    # and the objects still work afterwards
    rec = code.run_frames(1, "zero", 0, 0, 8, 1.0, 4)
    assert len(rec) == 8
