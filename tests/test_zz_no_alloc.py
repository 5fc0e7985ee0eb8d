"""The decode entry point that allocates no device memory.

Some callers of this library cannot call cudaMalloc: a host framework that owns every
byte of device memory through its own pool, or a real-time loop that forbids
allocation once it has started.  cb_decode_device_noalloc serves them by keeping the
decoder's scratch in a static device array.  This test calls it through the C ABI twice
in a row and checks both outputs against the allocating cb_decode_device on the same
LLRs.  The tolerance is zero: it is the same decoder, so the hard decisions and the
iteration counts must be identical.  The file's name makes pytest collect it last.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    dict(k=520, e=1040, bg=2, z=52, m=4, ebn0=1.0, precision="f64", n=96),
    dict(k=8448, e=25344, bg=1, z=384, m=16, ebn0=2.5, precision="f32", n=300),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['precision']}_z{c['z']}")
def test_no_alloc_decode_equals_the_allocating_decode(cb, case):
    import torch

    code = cb.NrLdpc(case["k"], case["e"], base_graph=case["bg"], lifting_size=case["z"],
                     precision=case["precision"])
    llr_host, _ = code.generate_frames(7, "no_alloc", 0, 0, case["n"], case["ebn0"], case["m"])
    dt = torch.float64 if case["precision"] == "f64" else torch.float32
    llr = torch.from_numpy(llr_host).to(device="cuda", dtype=dt)
    words = (case["k"] + 31) // 32
    n = case["n"]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = cb.lib()

    def run(fn):
        bits = torch.full((n, words), -1, dtype=torch.int32, device="cuda")
        iters = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        args = [code._h, C.c_void_p(llr.data_ptr()), n, C.c_void_p(bits.data_ptr())]
        if fn == "cb_decode_device":
            args.append(None)  # no a posteriori LLRs
        args += [C.c_void_p(iters.data_ptr()), stream]
        st = getattr(L, fn)(*args)
        assert st == 0, L.cb_last_error(code._h).decode()
        torch.cuda.synchronize()
        return bits.cpu().numpy(), iters.cpu().numpy()

    want_bits, want_iters = run("cb_decode_device")
    for _ in range(2):  # the scratch keeps the previous call's contents
        bits, iters = run("cb_decode_device_noalloc")
        assert np.array_equal(bits, want_bits)
        assert np.array_equal(iters, want_iters)
    assert (want_iters > 0).any()


def test_no_alloc_rejects_codes_it_cannot_serve(cb):
    code = cb.NrLdpc(500, 1200, rv=2, qm=4, precision="f32")  # rate matching with an offset k0
    with pytest.raises(cb.ComrsError) as ei:
        cb._check(cb.lib().cb_decode_device_noalloc(code._h, C.c_void_p(1), 1, None, None, None), code._h)
    assert ei.value.kind == "Config" and "plain rate matching" in str(ei.value)


def test_no_alloc_first_call_on_a_fresh_code_allocates_nothing(cb):
    # A code object whose first device call is cb_decode_device_noalloc: free device memory
    # (cudaMemGetInfo) is the same before and after two calls, the object does no device
    # set-up of its own, and the decisions equal the allocating decoder's.  A warm-up call
    # on another object first loads the library's kernels (the first launch of a module
    # maps its code into device memory; that is not an allocation by the entry point).
    import torch

    case = CASES[1]
    kw = dict(base_graph=case["bg"], lifting_size=case["z"], precision=case["precision"])
    warm = cb.NrLdpc(case["k"], case["e"], **kw)
    llr_host, _ = warm.generate_frames(7, "no_alloc_fresh", 0, 0, 64, case["ebn0"], case["m"])
    llr = torch.from_numpy(llr_host).to(device="cuda", dtype=torch.float32)
    n, words = 64, (case["k"] + 31) // 32
    L = cb.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    bits = torch.full((n, words), -1, dtype=torch.int32, device="cuda")
    iters = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    want_bits = torch.full((n, words), -1, dtype=torch.int32, device="cuda")
    want_iters = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    args = (C.c_void_p(llr.data_ptr()), n, C.c_void_p(bits.data_ptr()), C.c_void_p(iters.data_ptr()), stream)
    assert L.cb_decode_device_noalloc(warm._h, *args) == 0
    assert L.cb_decode_device(warm._h, C.c_void_p(llr.data_ptr()), n, C.c_void_p(want_bits.data_ptr()), None,
                              C.c_void_p(want_iters.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    want = (want_bits.cpu().numpy(), want_iters.cpu().numpy())
    bits.fill_(-1)
    iters.fill_(-1)
    torch.cuda.synchronize()
    fresh = cb.NrLdpc(case["k"], case["e"], **kw)
    for _ in range(2):
        free_before = torch.cuda.mem_get_info()[0]
        st = L.cb_decode_device_noalloc(fresh._h, *args)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert st == 0, L.cb_last_error(fresh._h).decode()
        assert free_after == free_before
        got = (bits.cpu().numpy(), iters.cpu().numpy())
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
        bits.fill_(-1)
        iters.fill_(-1)
        torch.cuda.synchronize()
    assert fresh.decoder == "not yet on a device"
