"""CPU pins of the label-propagation partition oracle, restated from the
reference's own unit tests (src/graph/label_prop.rs:571-739)."""
import numpy as np

import oracle as O


def test_iteration_skips_labelled_nodes():  # label_prop.rs:575-582
    assert list(O.lp_iteration([0, 1, 2, 3], [1, 0, 1], [1, 1, 1], [0, 1, 2])) == [0, 1, 2]


def test_iteration_propagates_strong_label():  # :584-592
    assert O.lp_iteration([0, 2, 2, 2], [1, 2], [2.0, 0.3], [-1, 5, 7])[0] == 5


def test_iteration_stays_unlabelled_below_threshold():  # :594-600
    assert O.lp_iteration([0, 1, 1], [1], [0.5], [-1, 3])[0] == -1


def test_iteration_ignores_unlabelled_neighbours():  # :602-609
    assert O.lp_iteration([0, 1, 1], [1], [5.0], [-1, -1])[0] == -1


def test_iteration_threshold_is_inclusive_and_last_tie_wins():
    # a total of exactly 1.0 ties the threshold and is accepted; of two equal
    # totals the label that appears last wins (label_prop.rs:69-83)
    assert O.lp_iteration([0, 1, 1], [1], [1.0], [-1, 4])[0] == 4
    assert O.lp_iteration([0, 2, 2, 2], [1, 2], [2.0, 2.0], [-1, 3, 9])[0] == 9
    # ties are ordered by first appearance, not by the last vote: label 3
    # appears first (1.5 + 0.5), label 9 second (2.0), so 9 wins
    assert O.lp_iteration([0, 3, 3, 3, 3], [1, 2, 3], [1.5, 2.0, 0.5], [-1, 3, 9, 3])[0] == 9


def test_outliers_finds_labelled_neighbour():  # :611-620
    lab = O.lp_outliers([0, 1, 3, 4], [1, 0, 2, 1], [-1, -1, 42], 99)
    assert lab[0] >= 0 and lab[1] == 42


def test_outliers_random_fallback_for_isolated():  # :622-630
    lab = O.lp_outliers([0, 0, 0], [], [-1, 5], 99)
    assert 0 <= lab[0] <= 5


def test_remap():  # :632-651
    lab, k = O.lp_remap([10, 10, 20, 20, 10])
    assert k == 2 and list(lab) == [0, 0, 1, 1, 0]
    lab, k = O.lp_remap([5, -1, 5, -1])
    assert k == 3 and lab[0] == 0 and lab[2] == 0 and {lab[1], lab[3]} == {1, 2}


def test_loop_returns_valid_partition():  # :653-680
    n = 5
    ip, ix = [0], []
    for i in range(n):
        ix += sorted({(i + 1) % n, (i - 1) % n})
        ip.append(len(ix))
    part, k = O.lp_partition(ip, ix, [1.0] * len(ix), 3, 10, 42)
    assert len(part) == n and k > 0 and np.all(part < k)
