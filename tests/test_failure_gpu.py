"""The bounded device-side wait and the status it reports (needs a GB300).

The large-owner kernel stages each owner chunk into shared memory with one bulk copy completed
on an mbarrier, and waits for it a bounded number of polls.  Here the first wait is told to give
up at once (ktri_opts.copy_wait_polls = KTRI_COPY_WAIT_NONE): the kernel then waits once more,
with the normal bound, so that the copy has landed before the block leaves, and reports the
timeout.  Nothing faults, traps or waits without a bound.  The call must fail with
KTRI_ERR_TIMEOUT and a total of 0, and the same context must then count exactly again -- the
status a host reads instead of the reference's MPI error exception (include/cetric/util.h:105-128)."""
import numpy as np
import pytest

from katric_gb300 import Config, KtriError, TriangleCounter, _native

pytestmark = pytest.mark.gpu


def _clique(k: int):
    fo = np.arange(k + 1, dtype=np.uint64) * (k - 1)
    head = np.array([u for v in range(k) for u in range(k) if u != v], dtype=np.uint32)
    return fo, head


def test_copy_wait_timeout_reports_and_context_recovers(oracle):
    torch = pytest.importorskip("torch")
    k = 400  # owners of out-degree up to 399 run in the large-owner kernel
    fo, head = _clique(k)
    expect = k * (k - 1) * (k - 2) // 6
    total, pv, _ = oracle.count(fo, head, num_threads=4)
    assert total == expect
    with TriangleCounter(0) as ctr:
        # host-buffer entry point: the status comes back from the call itself
        with pytest.raises(KtriError) as e:
            ctr.count(fo, head, Config(copy_wait_polls=_native.COPY_WAIT_NONE))
        assert e.value.code == _native.ERR_TIMEOUT
        t, p = ctr.count(fo, head, Config())
        assert t == expect and np.array_equal(p, pv)
        # device entry point: the status comes from ktri_ctx_check, and the total is 0
        dfo = torch.from_numpy(fo.view(np.int64)).cuda()
        dhd = torch.from_numpy(head.view(np.int32)).cuda()
        tot = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        dpv = torch.zeros(k, dtype=torch.int64, device="cuda")
        ctr.count_device(dfo.data_ptr(), dhd.data_ptr(), k, len(head), tot.data_ptr(), dpv.data_ptr(),
                         Config(copy_wait_polls=_native.COPY_WAIT_NONE))
        with pytest.raises(KtriError) as e:
            ctr.check()
        assert e.value.code == _native.ERR_TIMEOUT
        assert int(tot.item()) == 0
        ctr.count_device(dfo.data_ptr(), dhd.data_ptr(), k, len(head), tot.data_ptr(), dpv.data_ptr(), Config())
        ctr.check()
        assert int(tot.item()) == expect
        assert np.array_equal(dpv.cpu().numpy().view(np.uint64), pv)


def test_invalid_input_leaves_total_zero():
    """A device-side input error (a self-loop) also yields a total of 0, not another call's
    stale partial sums."""
    torch = pytest.importorskip("torch")
    fo = np.array([0, 2, 4, 6], dtype=np.uint64)
    head = np.array([1, 2, 0, 2, 0, 2], dtype=np.uint32)  # vertex 2 lists itself
    with TriangleCounter(0) as ctr:
        good_fo, good_head = _clique(50)
        ctr.count(good_fo, good_head)  # leaves nonzero partial sums in the workspace
        dfo = torch.from_numpy(fo.view(np.int64)).cuda()
        dhd = torch.from_numpy(head.view(np.int32)).cuda()
        tot = torch.full((1,), -1, dtype=torch.int64, device="cuda")
        ctr.count_device(dfo.data_ptr(), dhd.data_ptr(), 3, 6, tot.data_ptr(), None, Config())
        with pytest.raises(KtriError) as e:
            ctr.check()
        assert e.value.code == _native.ERR_INVALID_CSR
        assert int(tot.item()) == 0
