"""tg_time_pair_kernel / tg_pair_kernel_time: with timing on, each ordered
split-FP32 Acc and AccJerk call records exactly one pairwise-kernel launch
under its own kernel id (the bench's roofline is quoted on these events),
and nothing is recorded with timing off."""
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_pair_kernel_events_by_kernel():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tupan_gb300 import _native as N
    from tupan_gb300.ics import plummer_arrays
    n = 8192                                        # 2^26 pairs: the ordered path
    d = plummer_arrays(n, 1e-3, seed=3)
    T = {k: torch.tensor(v, dtype=torch.float64, device="cuda") for k, v in d.items()}
    outs = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(6)]
    f5 = [T[k].data_ptr() for k in ("mass", "rx", "ry", "rz", "eps2")]
    f8 = f5 + [T[k].data_ptr() for k in ("vx", "vy", "vz")]
    s = N.current_stream()

    def acc():
        N.call_device("acc", n, f5, n, f5, (), [o.data_ptr() for o in outs[:3]], N.PREC_DS32, s)

    def acc_jerk():
        N.call_device("acc_jerk", n, f8, n, f8, (), [o.data_ptr() for o in outs], N.PREC_DS32, s)

    prev = N.lib.tg_time_pair_kernel(1)
    try:
        N.pair_kernel_time(N.KERNEL_ACC)
        N.pair_kernel_time(N.KERNEL_ACC_JERK)
        acc(); acc_jerk(); acc_jerk()
        ms_a, n_a = N.pair_kernel_time(N.KERNEL_ACC)
        ms_j, n_j = N.pair_kernel_time(N.KERNEL_ACC_JERK)
        assert (n_a, n_j) == (1, 2)
        assert ms_a > 0 and ms_j > 0
        N.lib.tg_time_pair_kernel(0)
        acc(); acc_jerk()
        assert N.pair_kernel_time(N.KERNEL_ACC)[1] == 0 and N.pair_kernel_time(N.KERNEL_ACC_JERK)[1] == 0
    finally:
        N.lib.tg_time_pair_kernel(prev)
