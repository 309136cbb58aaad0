"""The hot path captured into a CUDA graph and replayed: clear, insert,
retrieve, erase, copy_if and the exclusive scan on one stream, with the
scratch given by the caller and the copy_if count left on the device, so
that no call allocates or synchronises while the stream is being captured.
Each replay must give the exact results of the eager calls (integer work:
the tolerance is zero)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_hot_path_replays_from_a_cuda_graph(hx):
    import torch
    from hashinator_gb300 import workloads
    n = 1 << 20
    keys, vals, q, _ = workloads.map_workload(n, 4, 77, erase_frac=0.0)
    er = keys[: n // 4]
    fill = np.uint32(0xA5A5A5A5)
    s = torch.cuda.Stream()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
    dk, dv, dq, de = dev(keys), dev(vals), dev(q), dev(er)
    out = torch.empty_like(dq)
    out2 = torch.empty_like(dq)
    x = dev(np.random.default_rng(5).integers(0, 2**32, size=3 * n + 7, dtype=np.uint64).astype(np.uint32))
    cout = torch.empty_like(x)
    dc = torch.zeros(1, dtype=torch.int64, device="cuda")
    y = (x & 15).contiguous()
    sout = torch.empty_like(y)
    nb_c = hx.tools.scratch_bytes(hx.SCRATCH_COPY_IF, x.numel())
    nb_s = hx.tools.scratch_bytes(hx.SCRATCH_SCAN, y.numel())
    sc_c = torch.empty(nb_c, dtype=torch.uint8, device="cuda")
    sc_s = torch.empty(nb_s, dtype=torch.uint8, device="cuda")
    m = hx.Hashmap(21, 4, stream=s)

    def work():
        out.fill_(int(fill.view(np.int32)))
        out2.fill_(int(fill.view(np.int32)))
        m.clear(stream=s)
        m.insert(dk, dv, target_lf=0.5, stream=s)
        m.retrieve(dq, out, stream=s)
        m.erase(de, stream=s)
        m.retrieve(dq, out2, stream=s)
        hx.tools.copy_if(x, cout, hx.Pred.mod_lt(100, 30), scratch=sc_c, scratch_bytes=nb_c, stream=s, d_count=dc)
        hx.tools.split_prefix_scan(y, sout, scratch=sc_s, scratch_bytes=nb_s, stream=s)

    want, _ = workloads.query_expectation(keys, vals, q, fill)
    gone = np.isin(q, er)
    want2 = want.copy()
    want2[gone] = fill
    xh = x.cpu().numpy().view(np.uint32)
    want_c = xh[(xh % np.uint32(100)) < 30]
    yh = y.cpu().numpy().view(np.uint32)
    want_s = np.zeros_like(yh)
    np.cumsum(yh[:-1], dtype=np.uint32, out=want_s[1:])

    def check():
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want)
        np.testing.assert_array_equal(out2.cpu().numpy().view(np.uint32), want2)
        c = int(dc.item())
        assert c == len(want_c)
        np.testing.assert_array_equal(cout[:c].cpu().numpy().view(np.uint32), want_c)
        np.testing.assert_array_equal(sout.cpu().numpy().view(np.uint32), want_s)

    with torch.cuda.stream(s):
        work()  # eager: first launches size every kernel's launch geometry
    check()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        work()
    for _ in range(3):
        out.zero_()
        out2.zero_()
        cout.zero_()
        sout.zero_()
        dc.zero_()
        torch.cuda.synchronize()
        g.replay()
        check()
    m.close()
