"""The comparator table of the bin-ordering kernel (k_order_bins, grid_build.cu) read from the
source and checked on the CPU: by the 0-1 principle (Knuth, TAOCP vol. 3, 5.3.4, exercise 11) a
comparator network that sorts every sequence of 0s and 1s sorts every sequence, so all 2^16
binary inputs of the 16-wide network are sorted here."""
import os
import re

import numpy as np

from conftest import ROOT


def _network():
    src = open(os.path.join(ROOT, "vare_gb300", "csrc", "grid_build.cu")).read()
    n = int(re.search(r"constexpr int kSortNet16 = (\d+);", src).group(1))
    body = re.search(r"kNet16\[2 \* kSortNet16\] = \{([^}]*)\}", src).group(1)
    vals = [int(v) for v in body.replace("\n", " ").split(",") if v.strip()]
    assert len(vals) == 2 * n
    return n, np.array(vals, np.int64).reshape(n, 2)


def test_network_pairs_are_ordered_and_in_range():
    n, pairs = _network()
    assert n == 63
    assert np.all(pairs[:, 0] < pairs[:, 1])
    assert np.all((pairs >= 0) & (pairs < 16))


def test_network_sorts_every_binary_input():
    _, pairs = _network()
    m = np.arange(1 << 16, dtype=np.int64)
    v = ((m[:, None] >> np.arange(16)) & 1).astype(np.int8)  # every 0-1 sequence, one per row
    for a, b in pairs:
        lo = np.minimum(v[:, a], v[:, b])
        hi = np.maximum(v[:, a], v[:, b])
        v[:, a], v[:, b] = lo, hi
    assert np.all(v[:, :-1] <= v[:, 1:])
