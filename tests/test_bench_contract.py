"""The roofline's algorithmic flop count follows the measurement contract:
F = sum over the decomposition's operations of per-order costs + N p + 2 N p
+ 2 N + 30, checked by hand for the Kepler system at order 19."""

import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_contract_flops_kepler_by_hand():
    import bench
    from hyk import workloads as W

    p, N = 19, 6
    orders = range(p + 1)
    # Kepler: 3 neg, 3 square, 2 add, 1 pow, 3 mul
    ops = 3 * (p + 1) + 3 * sum(n + 2 for n in orders) + 2 * (p + 1) + sum(4 * n + 3 for n in orders) + 3 * sum(
        2 * n + 1 for n in orders)
    assert bench.contract_flops(W.kepler_sys(), p) == ops + N * p + 2 * N * p + 2 * N + 30 == 3194


def test_contract_flops_sin_cos_pair_counted_once():
    import bench
    import hyk

    x, v = hyk.make_vars("x", "v")
    p = 20
    pair = sum(4 * n + 2 for n in range(p + 1)) + p
    one = bench.contract_flops([(x, v), (v, -9.8 * hyk.sin(x))], p)
    both = bench.contract_flops([(x, hyk.cos(x) * v), (v, -9.8 * hyk.sin(x))], p)
    assert both - one == sum(2 * n + 1 for n in range(p + 1))  # one more mul, the pair once
    assert one > pair
