"""Every traversal schedule and pattern tile of the mixed path gives the same
lnL (within the mixed tolerance, 1e-6 relative of the FP64 oracle), and for a
given kernel the fused, level-synchronous and dataflow schedules agree bit for
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
    for tile in (1, 2) + autotune.TILES:
        same_tile = [v for (t, _), v in got.items() if t == tile]
        assert len(set(same_tile)) <= 1, (tile, got)


def test_dna_dataflow_large(oracle_mod):
    """120-taxon DNA, 30,000 sites: hundreds of (op, tile) items whose children
    come from other CTAs of the same dataflow launch; bit-identical to the
    fused and level-synchronous launches of the same kernel."""
    from iqtree2_gb300 import simulate
    ds = simulate.dna_gtr_dataset(120, 30000, 51)
    topo = Topology(ds.edges, ds.lengths, ds.patterns.shape[0])
    eng = engine.Engine(ds.patterns.shape[1], ds.model.nstates, ds.model.ncat, ds.patterns.shape[0],
                        ds.model.state_unknown, topo.nslots, precision=engine.F32, max_ops=topo.nslots)
    eng.set_model(ds.model)
    eng.set_patterns(ds.freq)
    eng.set_tip_states(ds.patterns)
    leaf, nb = 0, topo.adj[0][0][0]
    ops = engine.Engine.ops_array(topo.branch_ops(nb, leaf))
    a, b, length = topo.ref(leaf, nb), topo.ref(nb, leaf), topo.edge_len(leaf, nb)
    want = oracle_mod.OracleTree(ds.model, ds.patterns, ds.freq, ds.edges, ds.lengths).lnl_branch(nb, leaf)
    got = []
    for cand in ((1, 0, 0, 0), (1, 1, 0, 0), (1, 2, 0, 0), (1, 2, 0, 0), (2, 1, 0, 0)):
        autotune.apply(eng, cand)
        got.append(eng.compute_likelihood(ops, a, b, length))
    assert len(set(got)) == 1, got
    assert rel(got[0], want) < 1e-6
