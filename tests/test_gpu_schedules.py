"""Every traversal schedule and pattern tile of the mixed path gives the same
lnL (within the mixed tolerance, 1e-6 relative of the FP64 oracle), and the
fused and level-synchronous schedules of the per-category kernel agree bit for
bit (same per-op arithmetic, different launch order)."""
import pytest

from helpers import load_golden, rel
from iqtree2_gb300 import autotune, engine
from iqtree2_gb300.topology import Topology

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["dna16", "prot12", "codon8"])
def test_all_schedules_agree(oracle_mod, name):
    g = load_golden(name)
    topo = Topology(g.edges, g.lengths, g.ntaxa)
    eng = engine.Engine(g.patterns.shape[1], g.model.nstates, g.model.ncat, g.ntaxa, g.model.state_unknown,
                        topo.nslots, precision=engine.F32, max_ops=topo.nslots)
    eng.set_model(g.model)
    eng.set_patterns(g.freq)
    eng.set_tip_states(g.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(g.model, g.patterns, g.freq, g.edges, g.lengths).lnl_branch(nb, leaf)
    got = {}
    for cand in autotune.candidates(eng):
        tile, sched = cand[0], cand[1]
        autotune.apply(eng, cand)
        got[(tile, sched)] = eng.compute_likelihood(ops, a, b, length)
        assert rel(got[(tile, sched)], want) < 1e-6, (tile, sched)
    for tile in (1,) + autotune.TILES:
        if (tile, 0) in got and (tile, 1) in got:
            assert got[(tile, 0)] == got[(tile, 1)]
