"""The committed scorer on held-out streams of the anytime-2m family
(2,000,000 transactions x 640 items, 3% floor; seeds 5010-5019): the final MFI
sets of the learned, canonical and plain (the reference's global
support-descending) orders are identical, and ordering each node's extensions
by the scorer reaches 95% of the final MFIs after about half the search nodes
of the plain order (geometric mean over the seeds; a count of nodes, so the
comparison does not depend on the clock)."""
import os

import numpy as np
import pytest

from sgfim import learned_order
from sgfim.engine import Engine

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "20261008-self-growing-evidence-agent_gb300", "sgfim", "data", "scorer_weights.npz")


def test_learned_order_reaches_95_percent_in_fewer_nodes():
    ratios, tree = [], []
    with Engine() as eng:
        learned_order.load_weights(eng, WEIGHTS)
        for seed in range(5010, 5020):
            eng.load_rows(learned_order.stream_rows(seed, 2_000_000))
            thr = int(np.ceil(0.03 * 2_000_000))
            plain = eng.mine(thr, order="support_desc")
            learned = eng.mine(thr, order="learned")
            assert learned.as_dict() == plain.as_dict()
            ratios.append(learned.nodes_to_coverage(0.95) / plain.nodes_to_coverage(0.95))
            tree.append(learned.nodes / plain.nodes)
    assert float(np.exp(np.mean(np.log(ratios)))) < 0.7
    assert float(np.exp(np.mean(np.log(tree)))) < 0.7
