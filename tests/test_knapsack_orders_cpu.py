"""The knapsack search orders on CPU (oracle/knapsack_orders.py): best-first,
breadth-first and the heap/FIFO switch all reach the capacity-DP optimum,
and on the GPU test's own instances (tests/test_batch_gpu.py) the model
gives what that test relies on: a switch counter of 2 makes each of the
four largest leave the heap once, and a counter of 1 brings them back
from the FIFO ring too."""
import numpy as np
import pytest

from oracle import knapsack_orders as ko
from oracle import pyoracle

pytest.importorskip("torch")
from gpuheap_gb300 import batch as gbb  # noqa: E402

FIFO_SIZES = (2, 17, 100, 200, 300, 500)  # tests/test_batch_gpu.py


@pytest.mark.parametrize("order,sizes", [("heap", (1, 3, 17, 40, 120)), ("switch", (1, 3, 17, 40, 120)),
                                         ("fifo", (1, 3, 10, 17, 25))])  # breadth-first grows fast
def test_every_order_reaches_the_optimum(order, sizes):
    for n in sizes:
        for seed in range(3):
            w, p, cap = gbb.gen_knapsack(n, 300 + 7 * n + seed)
            want = pyoracle.knap_dp(w, p, cap)
            for counter in (1, 2, 20):
                got, switches, _ = ko.search(w, p, cap, order, batch=64, counter=counter)
                assert got == want, (order, n, seed, counter)
                if order != "switch":
                    assert switches == 0


def test_switch_counts_on_the_gpu_test_instances():
    big = [gbb.gen_knapsack(n, 900 + n) for n in FIFO_SIZES[-4:]]
    for counter, want in ((2, 1), (1, 3)):
        got = []
        for w, p, cap in big:
            best, switches, _ = ko.search(w, p, cap, "switch", batch=128, counter=counter)
            assert best == pyoracle.knap_bb(w, p, cap)
            got.append(switches)
        assert got == [want] * 4, (counter, got)
