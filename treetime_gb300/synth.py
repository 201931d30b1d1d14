"""Seeded synthetic workloads: random trees, models and alignments evolved
down the tree.  They stand in for real data in tests and benchmarks; every
draw comes from one ``numpy.random.default_rng(seed)``.

Workloads (sizes as in the benchmark configurations):
  * ``c0``: Kingman-coalescent topology, 100 tips, branch lengths Exp(mean
    0.01); 1,000 nucleotide sites evolved from a uniform root under GTR with
    pi ~ Dirichlet(1,1,1,1) and symmetric exchangeabilities U(0.5, 2);
    alphabet 'nuc_nogap'; 5% of tip characters replaced by '-'.
  * ``c1``: coalescent, 2,000 tips, Exp(mean 5e-4); 30,000 sites, 90% of
    them invariant (the root state copied to every tip); GTR with
    transition/transversion ratio 3 and pi ~ Dirichlet(1,1,1,1).
  * ``c2``: Yule, 500 tips, Exp(mean 0.05); 1,500 amino-acid sites over a
    21-letter alphabet (20 amino acids + '-'); site-specific model with
    per-site pi ~ Dirichlet(0.5 × 21) and shared symmetric W ~ U(0.1, 5);
    no compression.
  * ``c3``: a batch of independent nucleotide trees with tip counts
    log-uniform in [50, 5000], site counts log-uniform in [1k, 30k], branch
    means log-uniform in [1e-4, 0.05], and a random GTR per tree.
"""

import numpy as np

from .alphabets import alphabets
from .gtr import GTR, GTR_site_specific
from .tree import Clade, Tree

AA21 = np.array(list("ACDEFGHIKLMNPQRSTVWY-"))


def coalescent_tree(n, mean_bl, rng, prefix="t"):
    """Kingman topology (uniformly random pair merges) with i.i.d.
    exponential branch lengths."""
    nodes = [Clade(branch_length=float(rng.exponential(mean_bl)), name="%s%d" % (prefix, i)) for i in range(n)]
    while len(nodes) > 1:
        i, j = rng.choice(len(nodes), size=2, replace=False)
        a, b = nodes[i], nodes[j]
        parent = Clade(branch_length=float(rng.exponential(mean_bl)), clades=[a, b])
        for k in sorted((i, j), reverse=True):
            nodes[k] = nodes[-1]
            nodes.pop()
        nodes.append(parent)
    root = nodes[0]
    root.branch_length = 0.001
    return Tree(root=root)


def yule_tree(n, mean_bl, rng, prefix="t"):
    """Yule topology (a uniformly random tip splits) with i.i.d. exponential
    branch lengths."""
    root = Clade(branch_length=0.001)
    tips = [root]
    while len(tips) < n:
        k = int(rng.integers(len(tips)))
        node = tips[k]
        a, b = Clade(), Clade()
        node.clades = [a, b]
        tips[k] = a
        tips.append(b)
    order = rng.permutation(n)
    for i, t in zip(order, tips):
        t.name = "%s%d" % (prefix, i)
    stack = [root]
    while stack:
        c = stack.pop()
        for ch in c.clades:
            ch.branch_length = float(rng.exponential(mean_bl))
            stack.append(ch)
    return Tree(root=root)


def _pmat(gtr, t):
    """Host P(t) for input generation only: columns are parent states."""
    e = np.exp(gtr.mu * gtr.eigenvals * t)
    return np.maximum(0.0, (gtr.v * e) @ gtr.v_inv)


def evolve(tree, gtr, L, rng, invariant_frac=0.0, root_states=None):
    """Evolve integer states from the root (uniform unless given) down the
    tree; returns {tip name: state indices}.  A fraction ``invariant_frac`` of
    sites keeps the root state everywhere."""
    q = gtr.n_states
    states = {}
    root = tree.root
    states[id(root)] = rng.integers(q, size=L) if root_states is None else np.asarray(root_states)
    variable = np.ones(L, dtype=bool)
    if invariant_frac > 0:
        variable[rng.random(L) < invariant_frac] = False
    var_idx = np.flatnonzero(variable)
    out = {}
    stack = [root]
    while stack:
        node = stack.pop()
        s = states.pop(id(node))
        if not node.clades:
            out[node.name] = s
            continue
        for ch in node.clades:
            P = _pmat(gtr, ch.branch_length)          # P[child, parent]
            cdf = np.cumsum(P.T, axis=1)               # rows: parent state
            cdf /= cdf[:, -1:]
            u = rng.random(len(var_idx))
            child = s.copy()
            sub = cdf[s[var_idx]]
            child[var_idx] = np.minimum((u[:, None] > sub).sum(axis=1), q - 1)
            states[id(ch)] = child
            stack.append(ch)
    return out


def evolve_sparse(tree, gtr, L, rng):
    """The same substitution process as ``evolve`` (uniform root), sampled per
    branch as "keep the parent state with probability P(s -> s), otherwise draw
    the new state from P(. | s) restricted to the other states": one uniform
    draw per site plus one per changed site, so short branches are cheap.
    Returns {tip name: uint8 state indices}."""
    q = gtr.n_states
    root = tree.root
    states = {id(root): rng.integers(q, size=L).astype(np.uint8)}
    out = {}
    stack = [root]
    while stack:
        node = stack.pop()
        s = states.pop(id(node))
        if not node.clades:
            out[node.name] = s
            continue
        for ch in node.clades:
            P = _pmat(gtr, ch.branch_length)               # P[child, parent]
            stay = np.diag(P).astype(np.float32)
            off = P.T.copy()                               # rows: parent state
            np.fill_diagonal(off, 0.0)
            tot = off.sum(axis=1, keepdims=True)
            cdf = np.cumsum(off / np.where(tot > 0, tot, 1.0), axis=1)
            u = rng.random(L, dtype=np.float32)
            moved = np.flatnonzero(u > stay[s])
            child = s.copy()
            if moved.size:
                v = rng.random(moved.size)
                child[moved] = np.minimum((v[:, None] > cdf[s[moved]]).sum(axis=1), q - 1).astype(np.uint8)
            states[id(ch)] = child
            stack.append(ch)
    return out


def c3_sizes(n_trees=256, seed=3, n_range=(50, 5000), L_range=(1000, 30000), bl_range=(1e-4, 0.05)):
    """(tips, sites, mean branch length) of every tree of ``forest_c3`` with
    the same arguments, without building any tree: each tree draws them first
    from its own generator."""
    out = []
    for k in range(n_trees):
        rng = np.random.default_rng([seed, k])
        lu = lambda lo, hi: float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        out.append((int(lu(*n_range)), int(lu(*L_range)), lu(*bl_range)))
    return out


def forest_c3(n_trees=256, seed=3, n_range=(50, 5000), L_range=(1000, 30000), bl_range=(1e-4, 0.05), only=None):
    """The batched workload as device-ready inputs: ``n_trees`` independent
    coalescent trees with tip counts, site counts and mean branch lengths
    log-uniform in the given ranges, each with its own random nucleotide GTR,
    alignments compressed to patterns.  Tree k draws everything from its own
    generator (seeded by (seed, k)), so any subset (``only``: tree indices)
    is built alone with the same result as in the whole batch.  Built from
    state codes directly (no alignment text).  Returns (inputs, gtrs), model
    index = position in the returned list."""
    from . import engine
    from .seqdata import compress_codes
    alpha = np.frombuffer("".join(alphabets["nuc_nogap"]).encode(), dtype=np.uint8)
    inputs, gtrs = [], []
    for k in (range(n_trees) if only is None else only):
        rng = np.random.default_rng([seed, k])
        lu = lambda lo, hi: float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        n = int(lu(*n_range))
        L = int(lu(*L_range))
        bl = lu(*bl_range)
        tree = coalescent_tree(n, bl, rng)
        gtr = GTR.random(mu=1.0, alphabet="nuc_nogap", rng=rng)
        st = evolve_sparse(tree, gtr, L, rng)
        layout = engine.TreeLayout(tree.root)
        tips = layout.nodes[layout.n_int:]
        codes = alpha[np.stack([st[t.name] for t in tips])]
        pc, mult, _, _ = compress_codes(codes, ord("N"))
        inputs.append(engine.TreeInput(layout, pc, np.arange(len(tips), dtype=np.int32), mult,
                                       engine.branch_lengths(layout, L), model=len(gtrs)))
        inputs[-1].tree = tree
        inputs[-1].full_length = L
        gtrs.append(gtr)
    return inputs, gtrs


def _to_text(states, alphabet, gap_frac, rng):
    alpha = np.asarray(alphabet)
    aln = {}
    for name in sorted(states, key=lambda s: int(s[1:]) if s[1:].isdigit() else s):
        chars = alpha[states[name]].copy()
        if gap_frac > 0:
            chars[rng.random(len(chars)) < gap_frac] = "-"
        aln[name] = "".join(chars.tolist())
    return aln


def gtr_c0(rng, alphabet="nuc_nogap"):
    n = len(alphabets[alphabet])
    pi = rng.dirichlet(np.ones(n))
    W = rng.uniform(0.5, 2.0, size=(n, n))
    W = np.triu(W, 1)
    W = W + W.T
    return GTR.custom(mu=1.0, pi=pi, W=W, alphabet=alphabet)


def gtr_c1(rng, kappa=3.0):
    pi = rng.dirichlet(np.ones(4))
    W = np.ones((4, 4))
    W[0, 2] = W[2, 0] = W[1, 3] = W[3, 1] = kappa
    return GTR.custom(mu=1.0, pi=pi, W=W, alphabet="nuc_nogap")


def gtr_c2(rng, L, approximate=True):
    n = len(AA21)
    pi = rng.dirichlet(np.full(n, 0.5), size=L).T
    W = rng.uniform(0.1, 5.0, size=(n, n))
    W = np.triu(W, 1)
    W = W + W.T
    gtr = GTR_site_specific(seq_len=L, approximate=approximate, alphabet=AA21)
    gtr.assign_rates(mu=1.0, pi=pi, W=W)
    return gtr


def make_workload(name, seed=0, **over):
    """Dict with ``tree``, ``aln`` (name -> string), ``gtr`` and the
    constructor options for one named workload.  Keyword overrides shrink
    sizes for tests (n, L, mean_bl, gap_frac, invariant_frac)."""
    rng = np.random.default_rng(seed)
    if name == "c0":
        n, L, bl = over.get("n", 100), over.get("L", 1000), over.get("mean_bl", 0.01)
        tree = coalescent_tree(n, bl, rng)
        gtr = over.get("gtr") or gtr_c0(rng, over.get("alphabet", "nuc_nogap"))
        states = evolve(tree, gtr, L, rng, invariant_frac=over.get("invariant_frac", 0.0))
        aln = _to_text(states, gtr.alphabet, over.get("gap_frac", 0.05), rng)
        return dict(tree=tree, aln=aln, gtr=gtr, compress=over.get("compress", True))
    if name == "c1":
        n, L, bl = over.get("n", 2000), over.get("L", 30000), over.get("mean_bl", 5e-4)
        tree = coalescent_tree(n, bl, rng)
        gtr = gtr_c1(rng)
        states = evolve(tree, gtr, L, rng, invariant_frac=over.get("invariant_frac", 0.9))
        aln = _to_text(states, gtr.alphabet, over.get("gap_frac", 0.0), rng)
        return dict(tree=tree, aln=aln, gtr=gtr, compress=True)
    if name == "c2":
        n, L, bl = over.get("n", 500), over.get("L", 1500), over.get("mean_bl", 0.05)
        tree = yule_tree(n, bl, rng)
        gtr = gtr_c2(rng, L, approximate=over.get("approximate", True))
        states = evolve_site_specific(tree, gtr, L, rng)
        aln = _to_text(states, gtr.alphabet, over.get("gap_frac", 0.0), rng)
        return dict(tree=tree, aln=aln, gtr=gtr, compress=False)
    if name == "c3":
        n_trees = over.get("n_trees", 256)
        jobs = []
        for k in range(n_trees):
            n = int(np.exp(rng.uniform(np.log(over.get("n_min", 50)), np.log(over.get("n_max", 5000)))))
            L = int(np.exp(rng.uniform(np.log(over.get("L_min", 1000)), np.log(over.get("L_max", 30000)))))
            bl = float(np.exp(rng.uniform(np.log(1e-4), np.log(0.05))))
            tree = coalescent_tree(n, bl, rng)
            gtr = GTR.random(mu=1.0, alphabet="nuc_nogap", rng=rng)
            states = evolve(tree, gtr, L, rng)
            aln = _to_text(states, gtr.alphabet, over.get("gap_frac", 0.0), rng)
            jobs.append(dict(tree=tree, aln=aln, gtr=gtr, compress=True))
        return dict(jobs=jobs)
    raise KeyError(name)


def evolve_site_specific(tree, gtr, L, rng):
    """Evolution under a site-specific model (per-site P(t))."""
    q = gtr.n_states
    lam, V, Vi = gtr.site_matrices()
    root = tree.root
    # root drawn from the per-site equilibrium frequencies
    cdf0 = np.cumsum(gtr.Pi.T, axis=1)
    root_states = np.minimum((rng.random(L)[:, None] > cdf0).sum(axis=1), q - 1)
    states = {id(root): root_states}
    out = {}
    stack = [root]
    sites = np.arange(L)
    while stack:
        node = stack.pop()
        s = states.pop(id(node))
        if not node.clades:
            out[node.name] = s
            continue
        for ch in node.clades:
            e = np.exp(gtr.mu[:, None] * lam * ch.branch_length)        # [L, q]
            # column of P_a[child, parent] at each site's parent state: V_a (e_a * V_a^-1[:, s_a])
            z = e * Vi[sites, :, s]                                        # [L, q] over eigen index
            col = np.maximum(np.matmul(V, z[:, :, None])[:, :, 0], 0.0)   # [L, q] over child states
            cdf = np.cumsum(col, axis=1)
            cdf /= cdf[:, -1:]
            child = np.minimum((rng.random(L)[:, None] > cdf).sum(axis=1), q - 1)
            states[id(ch)] = child
            stack.append(ch)
    return out
