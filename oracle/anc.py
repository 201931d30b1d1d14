"""Numpy restatement of TreeTime's ancestral-reconstruction and branch-length
hot path (TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``).

Every function follows the TreeTime 0.12.1 source cited in its docstring,
operation for operation (same reductions, same order of additions, the same
reciprocal-multiply normalisation), so that its FP64 results agree with the
reference to rounding.  Inputs are plain objects:

  tree   any rooted tree whose clades have ``.clades``, ``.name`` and
         ``.branch_length`` (optionally ``.mask``, a per-pattern array);
  model  any object with TreeTime's GTR attributes (``v``, ``v_inv``,
         ``eigenvals``, ``mu``, ``Pi``, ``alphabet``, ``profile_map``,
         ``gap_index``, ``is_site_specific`` and, site-specific,
         ``approximate``/``rate_scale``);
  aln    dict tip name -> compressed character array; ``mult`` the pattern
         multiplicities; ``full_length`` the uncompressed length.

Results are keyed by node name.
"""

import numpy as np

TINY_NUMBER = 1e-12
SUPERTINY_NUMBER = 1e-24
BIG_NUMBER = 1e10
MIN_BRANCH_LENGTH = 1e-3
MAX_BRANCH_LENGTH = 4.0


# ----------------------------------------------------------------- traversal
def preorder(root):
    stack = [root]
    while stack:
        n = stack.pop()
        yield n
        stack.extend(reversed(n.clades))


def postorder(root):
    stack = [(root, False)]
    while stack:
        n, done = stack.pop()
        if done or not n.clades:
            yield n
        else:
            stack.append((n, True))
            stack.extend((c, False) for c in reversed(n.clades))


def prepare_tree(tree, keep_node_order=False):
    """treeanc.py:446-510: root branch 0.001, ladderize (stable sort of each
    clade's children by tip count), name unnamed internal nodes NODE_%07d in
    preorder, set ``up`` links; branch lengths None -> 0 (treeanc.py:342-347)."""
    root = tree.root
    for n in preorder(root):
        n.branch_length = n.branch_length if n.branch_length else 0.0
        if not hasattr(n, "mask"):
            n.mask = None
    root.branch_length = 0.001
    root.mask = None
    if not keep_node_order:
        tips = {}
        for n in postorder(root):
            if n.clades:
                n.clades.sort(key=lambda c: tips[id(c)])
                tips[id(n)] = sum(tips[id(c)] for c in n.clades)
            else:
                tips[id(n)] = 1
    names = {n.name for n in preorder(root) if n.name}
    count = 0
    root.up = None
    for n in preorder(root):
        if not n.clades:
            continue
        if n.name is None:
            tmp = "NODE_" + format(count, "07d")
            while tmp in names:
                count += 1
                tmp = "NODE_" + format(count, "07d")
            n.name = tmp
            names.add(tmp)
        count += 1
        for c in n.clades:
            c.up = n
    return tree


def branch_length_to_gtr(node, full_length):
    """treeanc.py:752-760."""
    return max(MIN_BRANCH_LENGTH * (1.0 / full_length), node.branch_length)


# ----------------------------------------------------------------- model ops
def expQt(model, t):
    """gtr.py:1027-1067 (standard) and gtr_site_specific.py:331-371
    (site-specific, linear interpolation on the time grid when
    ``approximate``)."""
    if getattr(model, "is_site_specific", False):
        if t * model.rate_scale < 10 and model.approximate:
            from scipy.interpolate import interp1d
            grid = model.t_grid
            return interp1d(grid, _site_stack(model), axis=0, assume_sorted=True, copy=False, kind="linear")(t)
        return _site_expQt_exact(model, t)
    log_val = model.mu * t * model.eigenvals
    if any(i > 10 for i in log_val):
        raise ValueError("Error in computing exp(Q * t)")
    e = np.exp(log_val)
    Qs = model.v.dot(np.diag(e).dot(model.v_inv))
    return np.maximum(0, Qs)


def expQt_expm1(model, t):
    """exp(Qt) as I + V diag(expm1(mu lam t)) V^-1, clipped at 0: the same
    matrix as expQt (standard models), but with the small off-diagonal entries
    of short times accurate to rounding relative to their own size instead of
    set by the rounding of V diag(exp) V^-1 (exactly 0 at t = 0)."""
    em1 = np.expm1(model.mu * t * model.eigenvals)
    return np.maximum(0, np.eye(len(em1)) + model.v.dot(np.diag(em1).dot(model.v_inv)))


def _site_stack(model):
    """The exact per-site matrices at the grid points that TreeTime's
    interpolator is built from (gtr_site_specific.py:331-348), computed once
    per model object (TreeTime builds its interpolator once too)."""
    key = (id(model.v), id(model.v_inv), id(model.eigenvals), id(model.mu), id(model.t_grid))
    hit = getattr(model, "_oracle_stack", None)
    if hit is None or hit[0] != key:
        hit = (key, np.stack([_site_expQt_exact(model, tk) for tk in model.t_grid], axis=0))
        try:
            model._oracle_stack = hit
        except AttributeError:
            pass
    return hit[1]


def _site_expQt_exact(model, t):
    """gtr_site_specific.py:350-365 (no clamp)."""
    e = np.exp(t * model.mu * model.eigenvals)
    return np.einsum("jia,ja,kja->ika", model.v, e, model.v_inv)


def propagate_profile(model, profile, t, return_log=False):
    """gtr.py:965-995; gtr_site_specific.py:376-406."""
    Qt = expQt(model, t)
    if getattr(model, "is_site_specific", False):
        res = np.einsum("ai,ija->aj", profile, Qt)
        return np.log(np.maximum(TINY_NUMBER, res)) if return_log else np.maximum(0, res)
    res = profile.dot(Qt)
    return np.log(res) if return_log else res


def evolve(model, profile, t, return_log=False):
    """gtr.py:997-1025; gtr_site_specific.py:408-437."""
    Qt = expQt(model, t)
    if getattr(model, "is_site_specific", False):
        res = np.einsum("ai,jia->aj", profile, Qt)
    else:
        res = profile.dot(Qt.T)
    return np.log(res) if return_log else res


def normalize_profile(in_profile, log=False, return_offset=True):
    """seq_utils.py:279-307: rows scaled by the reciprocal of their sum."""
    if log:
        pre = in_profile.max(axis=1)
        tmp = np.exp(in_profile.T - pre).T
    else:
        pre = 0.0
        tmp = in_profile
    norm = tmp.sum(axis=1)
    return np.einsum("ai,a->ai", tmp, 1.0 / norm), (np.log(norm) + pre) if return_offset else None


def seq2prof(seq, profile_map):
    """seq_utils.py:207-229."""
    return np.array([profile_map[k] for k in seq])


def prof2seq(profile, model, sample_from_prof=False, normalize=True, rng=None):
    """seq_utils.py:232-276: first-index argmax, or inverse-CDF sampling with
    one ``rng.random(L)`` draw."""
    tmp = normalize_profile(profile, return_offset=False)[0] if normalize else profile
    if sample_from_prof:
        cumdis = tmp.cumsum(axis=1).T
        r = rng.random(size=cumdis.shape[1])
        idx = np.argmax(cumdis >= r, axis=0)
    else:
        idx = tmp.argmax(axis=1)
    seq = model.alphabet[idx]
    return seq, tmp[np.arange(tmp.shape[0]), idx], idx


def _pi_rows(model, L):
    Pi = np.asarray(model.Pi)
    return np.repeat([Pi], L, axis=0) if Pi.ndim == 1 else np.copy(Pi.T)


# ------------------------------------------------------------------ marginal
def marginal(tree, aln, mult, model, full_length, sample_from_profile=False, reconstruct_tip_states=False,
             rng=None, prev_cseq=None):
    """TreeAnc._ml_anc_marginal (treeanc.py:762-812) with
    postorder_traversal_marginal (:840-878), total_LH_and_root_sequence
    (:814-838) and preorder_traversal_marginal (:880-932).

    Returns dict with per-node ``subtree_LH``, ``outgroup_LH``, ``profile``,
    ``cseq`` and tree-level ``sequence_LH``, ``total_sequence_LH``, ``N_diff``.
    ``prev_cseq`` (name -> chars) plays the role of an earlier
    reconstruction; None means none existed.
    """
    L = len(mult)
    q = len(model.alphabet)
    root = tree.root
    bl = lambda n: branch_length_to_gtr(n, full_length)
    sub, pref, logLx, out, prof, cseq = {}, {}, {}, {}, {}, {}
    for leaf in (n for n in preorder(root) if not n.clades):
        sub[leaf.name] = seq2prof(aln[leaf.name], model.profile_map) if leaf.name in aln else np.ones((L, q))
        pref[leaf.name] = np.zeros(L)
    for node in (n for n in postorder(root) if n.clades):
        tmp = np.zeros((L, q), dtype=float)
        pref[node.name] = np.zeros(L, dtype=float)
        for ch in node.clades:
            lx = propagate_profile(model, sub[ch.name], bl(ch), return_log=True)
            if getattr(ch, "mask", None) is not None:
                lx = (lx.T * ch.mask).T
            logLx[ch.name] = lx
            tmp += lx
            pref[node.name] += pref[ch.name]
        sub[node.name], off = normalize_profile(tmp, log=True)
        pref[node.name] += off
    if sample_from_profile == "root":
        root_sample, other_sample = True, False
    else:
        root_sample = other_sample = bool(sample_from_profile)
    out[root.name] = _pi_rows(model, L)
    prof[root.name], pre = normalize_profile(out[root.name] * sub[root.name])
    seq_lh = pref[root.name] + pre
    total = (seq_lh * mult).sum()
    cseq[root.name] = prof2seq(prof[root.name], model, sample_from_prof=root_sample, normalize=False, rng=rng)[0]
    n_diff = 0
    for node in preorder(root):
        if node is root:
            continue
        parent = node.up
        out[node.name] = normalize_profile(
            np.log(np.maximum(TINY_NUMBER, prof[parent.name])) - logLx[node.name], log=True, return_offset=False)[0]
        if not node.clades and not reconstruct_tip_states:
            continue
        msg = evolve(model, out[node.name], bl(node), return_log=False)
        mask = getattr(node, "mask", None)
        if mask is None:
            prof[node.name] = normalize_profile(sub[node.name] * msg, return_offset=False)[0]
        else:
            prof[node.name] = normalize_profile(sub[node.name] * (mask * msg.T + (1.0 - mask)).T,
                                                return_offset=False)[0]
        seq = prof2seq(prof[node.name], model, sample_from_prof=other_sample, normalize=False, rng=rng)[0]
        if prev_cseq is not None:
            n_diff += int((seq != prev_cseq[node.name]).sum())
        else:
            n_diff += L
        cseq[node.name] = seq
    return dict(subtree_LH=sub, outgroup_LH=out, profile=prof, cseq=cseq, log_Lx=logLx,
                sequence_LH=seq_lh, total_sequence_LH=total, N_diff=n_diff)


# --------------------------------------------------------------------- joint
def joint(tree, aln, mult, model, full_length, sample_from_profile=False, reconstruct_tip_states=False,
          rng=None, prev_cseq=None):
    """TreeAnc._ml_anc_joint (treeanc.py:934-1080).  Also returns, per node,
    the top-two margin of the max-product choice for each parent state
    (``margin``) so that callers can exclude near-ties."""
    L = len(mult)
    q = len(model.alphabet)
    root = tree.root
    bl = lambda n: branch_length_to_gtr(n, full_length)
    Lx, Cx, margin = {}, {}, {}
    for node in postorder(root):
        if node is root:
            continue
        logT = np.log(np.maximum(TINY_NUMBER, expQt(model, bl(node))))
        if not node.clades:
            if node.name in aln:
                tmp = seq2prof(aln[node.name], model.profile_map)
                msg = np.log(np.maximum(tmp, TINY_NUMBER))
            else:
                msg = np.zeros((L, q))
            msg[np.isnan(msg) | np.isinf(msg)] = -BIG_NUMBER
        else:
            msg = np.sum(np.stack([Lx[c.name] for c in node.clades], axis=0), axis=0)
        lx = np.zeros((L, q))
        cx = np.zeros((L, q), dtype=np.uint16)
        mg = np.zeros((L, q))
        mask = getattr(node, "mask", None)
        for j in range(q):
            if mask is None:
                m = logT[:, j].T + msg
            else:
                m = (logT[:, j] * np.repeat([mask], q, axis=0).T) + msg
            cx[:, j] = m.argmax(axis=1)
            lx[:, j] = m.max(axis=1)
            srt = np.sort(m, axis=1)
            mg[:, j] = srt[:, -1] - srt[:, -2] if q > 1 else np.inf
            if mask is not None:
                lx[:, j] *= mask
        Lx[node.name], Cx[node.name], margin[node.name] = lx, cx, mg
    msg = np.sum(np.stack([Lx[c.name] for c in root.clades], axis=0), axis=0)
    root_lx = msg + np.log(model.Pi).T
    normalized = (root_lx.T - root_lx.max(axis=1)).T
    srt = np.sort(root_lx, axis=1)
    root_margin = srt[:, -1] - srt[:, -2]
    root_sample = True if sample_from_profile == "root" else bool(sample_from_profile)
    seq, _, idxs = prof2seq(np.exp(normalized), model, sample_from_prof=root_sample, rng=rng)
    seq_lh = np.choose(idxs, root_lx.T)
    total = (seq_lh * mult).sum()
    cseq = {root.name: seq}
    seq_idx = {root.name: idxs}
    n_diff = 0
    nodes = [n for n in preorder(root) if n.clades]
    if reconstruct_tip_states:
        nodes += [n for n in preorder(root) if not n.clades]
    for node in nodes:
        if node is root:
            continue
        seq_idx[node.name] = np.choose(seq_idx[node.up.name], Cx[node.name].T)
        s = np.choose(seq_idx[node.name], model.alphabet)
        if prev_cseq is not None:
            n_diff += int((s != prev_cseq[node.name]).sum())
        else:
            n_diff += L
        cseq[node.name] = s
    return dict(cseq=cseq, seq_idx=seq_idx, joint_Lx=Lx, joint_Cx=Cx, margin=margin, root_margin=root_margin,
                root_Lx=root_lx, sequence_LH=seq_lh, sequence_joint_LH=total, N_diff=n_diff)


def fitch(tree, tip_cseq, L, rng, prev_cseq=None):
    """TreeAnc._fitch_anc (treeanc.py:575-643) with _fitch_state (:645-664)
    and _fitch_intersect (:666-686): Python lists of characters per node and
    position.  ``tip_cseq`` name -> compressed characters; returns (name ->
    characters of every internal node, N_diff)."""
    state = {}
    for leaf in (n for n in preorder(tree.root) if not n.clades):
        state[leaf.name] = [[k] for k in tip_cseq[leaf.name]]

    def intersect(arrays):
        arrays = list(arrays)
        while len(arrays) > 1:
            arr1 = arrays.pop()
            s2 = set(arrays.pop())
            arrays.append([v for v in arr1 if v in s2])
        return arrays[0]

    for node in (n for n in postorder(tree.root) if n.clades):
        st = []
        for pos in range(L):
            s = intersect([state[c.name][pos] for c in node.clades])
            if len(s) == 0:
                s = list(np.concatenate([state[c.name][pos] for c in node.clades]))
            st.append(s)
        state[node.name] = st
    cseq = {tree.root.name: np.array([k[rng.integers(len(k)) if len(k) > 1 else 0] for k in state[tree.root.name]])}
    n_diff = 0
    for node in preorder(tree.root):
        if not node.clades or node is tree.root:
            continue
        par = cseq[node.up.name]
        seq = np.array([par[i] if par[i] in state[node.name][i] else state[node.name][i][0] for i in range(L)])
        if prev_cseq is not None:
            n_diff += int((seq != prev_cseq[node.name]).sum())
        else:
            n_diff += L
        cseq[node.name] = seq
    return cseq, n_diff


def ancestral_likelihood(tree, cseq, mult, model, full_length):
    """TreeAnc.ancestral_likelihood (treeanc.py:714-750): per-pattern log-LH
    of a full assignment of sequences."""
    log_lh = np.zeros(len(mult))
    idx = {s: i for i, s in enumerate(model.alphabet)}
    for node in postorder(tree.root):
        if node is tree.root:
            p = seq2prof(cseq[node.name], model.profile_map) * model.Pi
            log_lh += np.log(p.sum(axis=1))
            continue
        ind = np.array([(idx[a], idx[b]) for a, b in zip(cseq[node.up.name], cseq[node.name])])
        logQt = np.log(expQt(model, node.branch_length))
        log_lh += logQt[ind[:, 1], ind[:, 0]]
    return log_lh


# ------------------------------------------------------------ branch lengths
def state_pair(model, seq_p, seq_ch, pattern_multiplicity=None, ignore_gaps=False):
    """gtr.py:631-712, both the small-alphabet (boolean masks) and the
    large-alphabet (index loop, unknown -> 1) branches."""
    from collections import defaultdict
    if pattern_multiplicity is None:
        pattern_multiplicity = np.ones_like(seq_p, dtype=float)
    if seq_ch.shape != seq_p.shape:
        raise ValueError("GTR.state_pair: Sequence lengths do not match!")
    alphabet = model.alphabet
    gap = model.gap_index
    if len(alphabet) < 10:
        pair_count = []
        bp = [seq_p == c for c in alphabet]
        bc = [seq_ch == c for c in alphabet]
        for n1 in range(len(alphabet)):
            if gap is None or not ignore_gaps or n1 != gap:
                for n2 in range(len(alphabet)):
                    if gap is None or not ignore_gaps or n2 != gap:
                        count = ((bp[n1] & bc[n2]) * pattern_multiplicity).sum()
                        if count:
                            pair_count.append(((n1, n2), count))
    else:
        num = []
        for seq in (seq_p, seq_ch):
            tmp = np.ones_like(seq, dtype=int)
            for ni, c in enumerate(alphabet):
                tmp[seq == c] = ni
            num.append(tmp)
        pc = defaultdict(int)
        for i in range(len(seq_p)):
            if not ignore_gaps or (gap != num[0][i] and gap != num[1][i]):
                pc[(num[0][i], num[1][i])] += pattern_multiplicity[i]
        pair_count = pc.items()
    return (np.array([x[0] for x in pair_count], dtype=int),
            np.array([x[1] for x in pair_count], dtype=int))


def prob_t_compressed(model, seq_pair, multiplicity, t, return_log=False):
    """gtr.py:717-749."""
    if t < 0:
        logP = -BIG_NUMBER
    else:
        logQt = np.log(np.maximum(expQt(model, t), SUPERTINY_NUMBER))
        logP = np.sum(logQt[seq_pair[:, 1], seq_pair[:, 0]] * multiplicity)
    return logP if return_log else np.exp(logP)


def prob_t_profiles(model, profile_pair, multiplicity, t, return_log=False, ignore_gaps=True):
    """gtr.py:922-963."""
    if t < 0:
        logP = -BIG_NUMBER
    else:
        Qt = expQt(model, t)
        if len(Qt.shape) == 3:
            res = np.einsum("ai,ija,aj->a", profile_pair[1], Qt, profile_pair[0])
        else:
            res = np.einsum("ai,ij,aj->a", profile_pair[1], Qt, profile_pair[0])
        if ignore_gaps and model.gap_index is not None:
            ngf = (1 - profile_pair[0][:, model.gap_index]) * (1 - profile_pair[1][:, model.gap_index])
            logP = np.sum(multiplicity * np.log(res + SUPERTINY_NUMBER) * ngf)
        else:
            logP = np.sum(multiplicity * np.log(res + SUPERTINY_NUMBER))
    return logP if return_log else np.exp(logP)


def optimal_t_compressed(model, seq_pair, multiplicity, profiles=False, tol=1e-10):
    """gtr.py:816-920: scipy Brent over s = sqrt(t) with bracket
    (-sqrt(4), sqrt(hamming), sqrt(4)); Hamming distance if not successful.
    Returns (t, info) where info carries the Brent result."""
    from scipy.optimize import minimize_scalar

    def neg(s):
        if profiles:
            return -1.0 * prob_t_profiles(model, seq_pair, multiplicity, s ** 2, return_log=True) + np.exp(s ** 4 / 10000)
        return -1.0 * prob_t_compressed(model, seq_pair, multiplicity, s ** 2, return_log=True)

    if profiles:
        hamming = 1 - np.sum(multiplicity * np.sum(seq_pair[0] * seq_pair[1], axis=1)) / np.sum(multiplicity)
    else:
        hamming = np.sum(multiplicity[seq_pair[:, 1] != seq_pair[:, 0]]) / np.sum(multiplicity)
    opt = minimize_scalar(neg, bracket=[-np.sqrt(MAX_BRANCH_LENGTH), np.sqrt(hamming), np.sqrt(MAX_BRANCH_LENGTH)],
                          tol=tol, method="brent")
    new_len = opt["x"] ** 2
    if opt["success"] is not True:
        new_len = hamming
    return new_len, opt


def branch_len_grid(mutation_length, one_mutation, n_grid_points=125):
    """BranchLenInterpolator's grid, branch_len_interpolator.py:36-62."""
    if mutation_length < np.min((1e-5, 0.1 * one_mutation)):
        short_range = 10 * one_mutation
        return np.concatenate([short_range * (np.linspace(0, 1.0, n_grid_points // 2)[:-1]),
                               short_range + (MAX_BRANCH_LENGTH - short_range)
                               * (np.linspace(0, 1.0, n_grid_points // 2 + 1) ** 2)])
    sigma = mutation_length
    grid_left = mutation_length * (1 - np.linspace(1, 0.0, n_grid_points // 3) ** 2.0)
    grid_zero = grid_left[1] * np.logspace(-20, 0, 6)[:5]
    grid_zero2 = grid_left[1] * np.linspace(0, 1, 10)[1:-1]
    grid_right = mutation_length + (3 * sigma * (np.linspace(0, 1, n_grid_points // 3) ** 2))
    far_grid = grid_right.max() + MAX_BRANCH_LENGTH * np.linspace(0, 1, n_grid_points // 3) ** 2
    grid = np.concatenate((grid_zero, grid_zero2, grid_left, grid_right[1:], far_grid[1:]))
    grid.sort()
    return grid


def branch_len_log_prob(model, grid, mode, profile_pair=None, multiplicity=None, seq_pair=None,
                        pair_multiplicity=None, expm1_form=False):
    """-log P on the grid, branch_len_interpolator.py:103-118 ('marginal':
    prob_t_profiles of the branch's profile pair; 'joint': prob_t_compressed
    of its state pairs).  ``expm1_form``: 'joint' values from expQt_expm1."""
    if mode == "marginal":
        return np.array([-prob_t_profiles(model, profile_pair, multiplicity, k, return_log=True) for k in grid])
    if expm1_form:
        out = []
        for k in grid:
            logQt = np.log(np.maximum(expQt_expm1(model, k), SUPERTINY_NUMBER))
            out.append(BIG_NUMBER if k < 0 else -np.sum(logQt[seq_pair[:, 1], seq_pair[:, 0]] * pair_multiplicity))
        return np.array(out)
    return np.array([-prob_t_compressed(model, seq_pair, pair_multiplicity, k, return_log=True) for k in grid])


def pair_resolution(model, grid, seq_pair):
    """Per grid point, the smallest exp(Qt) entry (expQt_expm1) over the
    observed state pairs: where it is below ~1e-6 the reference's own value
    is dominated by the rounding of V diag(exp) V^-1."""
    return np.array([np.min(expQt_expm1(model, k)[seq_pair[:, 1], seq_pair[:, 0]]) if len(seq_pair) else 1.0
                     for k in grid])


def branch_mutation_matrix(model, pp, pc, t):
    """treeanc.py:1085-1120: normalised pc_i pp_j (expQt(t)_ij + 1e-24) per
    pattern, [L, q, q] (site-specific models: the pattern's own expQt)."""
    Qt = expQt(model, t) + SUPERTINY_NUMBER
    if Qt.ndim == 3:
        M = np.einsum("ai,aj,ija->aij", pc, pp, Qt)
    else:
        M = np.einsum("ai,aj,ij->aij", pc, pp, Qt)
    norm = M.sum(axis=2).sum(axis=1)
    return np.einsum("aij,a->aij", M, 1.0 / norm)


def substitution_counts_marginal(tree, res, mult, model, full_length):
    """The 'marginal' counting loop of TreeAnc.infer_gtr (treeanc.py:1544-1563)
    from an oracle marginal reconstruction ``res``: (n_ija, T_ia)."""
    q = len(model.alphabet)
    L = len(mult)
    n_ija = np.zeros((q, q, L))
    T_ia = np.zeros((q, L))
    for node in preorder(tree.root):
        if not node.clades:
            continue
        for c in node.clades:
            t = branch_length_to_gtr(c, full_length)
            mut = np.transpose(branch_mutation_matrix(model, res["outgroup_LH"][c.name], res["subtree_LH"][c.name],
                                                      t), (1, 2, 0))
            m = mult if getattr(c, "mask", None) is None else mult * c.mask
            T_ia += 0.5 * t * mut.sum(axis=0) * m
            T_ia += 0.5 * t * mut.sum(axis=1) * m
            n_ija += mut * m
    return n_ija, T_ia


def substitution_counts_joint(tree, cseq, raw_of, f2c, mult, model, full_length):
    """The 'joint' counting loop of TreeAnc.infer_gtr (treeanc.py:1564-1582):
    mutations on the full-length sequences (a tip's raw characters when
    ``raw_of(name)`` gives them, else its compressed sequence), skipped where a
    character is not a state; ``cseq`` name -> compressed characters."""
    q = len(model.alphabet)
    L = len(mult)
    index = {s: i for i, s in enumerate(np.asarray(model.alphabet).tolist())}
    n_ija = np.zeros((q, q, L))
    T_ia = np.zeros((q, L))
    for node in preorder(tree.root):
        if not node.clades:
            continue
        for c in node.clades:
            t = branch_length_to_gtr(c, full_length)
            parent = cseq[node.name][f2c]
            raw = raw_of(c.name)
            child = raw if raw is not None else (cseq[c.name][f2c] if c.name in cseq else None)
            if child is not None:
                for pos in np.where(parent != child)[0]:
                    a, d = parent[pos], child[pos]
                    if a not in index or d not in index:
                        continue
                    i, j = index[d], index[a]
                    cpos = f2c[pos]
                    n_ija[i, j, cpos] += 1
                    T_ia[j, cpos] += 0.5 * t
                    T_ia[i, cpos] -= 0.5 * t
            if c.name in cseq:
                m = mult if getattr(c, "mask", None) is None else mult * c.mask
                for i, nuc in enumerate(model.alphabet):
                    ind = cseq[c.name] == nuc
                    T_ia[i, ind] += t * m[ind]
    return n_ija, T_ia


def optimize_branch_lengths_joint(tree, cseq_of, mult, model, ignore_gaps=True):
    """TreeAnc.optimize_branch_lengths_joint (treeanc.py:1176-1242) with
    optimal_branch_length (:1244-1270) and add_branch_state (:1148-1163).
    ``cseq_of(node)`` returns the node's compressed sequence.  Returns
    name -> new length (branch lengths are not modified)."""
    out = {}
    for node in postorder(tree.root):
        if node is tree.root:
            continue
        m = mult if getattr(node, "mask", None) is None else mult * node.mask
        pairs, pm = state_pair(model, cseq_of(node.up), cseq_of(node), pattern_multiplicity=m, ignore_gaps=ignore_gaps)
        t, _ = optimal_t_compressed(model, pairs, pm)
        out[node.name] = max(0, t)
    return out


def optimize_tree_marginal(tree, aln, mult, model, full_length, max_iter=10, damping=0.75, LHtol=0.1):
    """TreeAnc.optimize_tree_marginal (treeanc.py:1297-1360) without GTR
    inference: marginal reconstruction, then per iteration i every branch's
    profile-mode Brent (tolerance 1e-8 + 0.01^(i+1)) with the damped update
    new*(1 - damping^(i+1)) + old*damping^(i+1), in TreeTime's preorder visit;
    the two children of a bifurcating root form one branch (parent profile
    normalize(subtree(n2) * outgroup(root))), updated at the visit of each
    child (:1318-1341).  Stops when the log-likelihood gains less than LHtol.
    Branch (and mutation) lengths of ``tree`` are updated in place.  Returns
    (last marginal result, per-iteration total log-likelihoods)."""
    res = marginal(tree, aln, mult, model, full_length)
    old_lh = res["total_sequence_LH"]
    history = []
    root = tree.root
    for i in range(max_iter):
        tol = 1e-8 + 0.01 ** (i + 1)
        d = damping ** (i + 1)
        for n in preorder(root):
            if n is root:
                continue
            if n.up is root and len(root.clades) == 2:
                n1, n2 = root.clades
                total_bl = n1.branch_length + n2.branch_length
                bl_ratio = n1.branch_length / total_bl
                prof_c = res["subtree_LH"][n1.name]
                prof_p = normalize_profile(res["subtree_LH"][n2.name] * res["outgroup_LH"][root.name])[0]
                m1, m2 = getattr(n1, "mask", None), getattr(n2, "mask", None)
                m = mult if m1 is None or m2 is None else mult * (m1 * m2)
                new_bl, _ = optimal_t_compressed(model, (prof_p, prof_c), m, profiles=True, tol=tol)
                update = new_bl * (1 - d) + total_bl * d
                n1.branch_length = update * bl_ratio
                n2.branch_length = update * (1 - bl_ratio)
                n1.mutation_length = n1.branch_length
                n2.mutation_length = n2.branch_length
            else:
                mask = getattr(n, "mask", None)
                m = mult if mask is None else mult * mask
                new_val, _ = optimal_t_compressed(model, (res["outgroup_LH"][n.name], res["subtree_LH"][n.name]), m,
                                                  profiles=True, tol=tol)
                n.branch_length = new_val * (1 - d) + n.branch_length * d
                n.mutation_length = n.branch_length
        res = marginal(tree, aln, mult, model, full_length)
        lh = res["total_sequence_LH"]
        history.append(lh)
        delta = lh - old_lh
        old_lh = lh
        if delta < LHtol:
            break
    return res, history


def prune_short_branches(tree, cseq_of, mult, model, one_mutation):
    """TreeAnc.prune_short_branches (treeanc.py:1475-1497): in preorder, an
    internal branch shorter than 0.1 * one_mutation whose parent and child
    sequences have probability > 0.1 at distance zero (GTR.prob_t: state
    pairs with gaps ignored, the node's mask on the multiplicities) is
    collapsed, its children re-attached to its parent; a node visited after
    its parent was collapsed is compared with its new parent.  Modifies
    ``tree``; returns the names of the collapsed nodes."""
    out = []
    for node in preorder(tree.root):
        if node.up is None or not node.clades:
            continue
        if node.branch_length < 0.1 * one_mutation:
            mask = getattr(node, "mask", None)
            m = mult if mask is None else mult * mask
            pairs, pm = state_pair(model, cseq_of(node.up), cseq_of(node), pattern_multiplicity=m, ignore_gaps=True)
            if prob_t_compressed(model, pairs, pm, 0.0) > 0.1:
                node.up.clades = [k for k in node.up.clades if k != node] + node.clades
                for clade in node.clades:
                    clade.up = node.up
                out.append(node.name)
    return out


def optimize_tree_joint(tree, aln, mult, model, full_length, one_mutation, max_iter=5, prune_short=True):
    """TreeAnc.optimize_tree with branch_length_mode='joint' (treeanc.py:
    1384-1473): joint reconstruction, joint branch lengths, then up to
    max_iter rounds of (pruning of short branches, joint reconstruction; stop
    when no character changed; joint branch lengths).  Branch lengths and the
    topology of ``tree`` are updated in place.  Returns (last joint result,
    unconstrained_sequence_LH)."""
    def cseq_of(cseq):
        return lambda n: cseq[n.name] if n.clades or n.name not in aln else aln[n.name]

    def set_lengths(res):
        new = optimize_branch_lengths_joint(tree, cseq_of(res["cseq"]), mult, model)
        for n in postorder(tree.root):
            if n is not tree.root:
                n.branch_length = new[n.name]
                n.mutation_length = new[n.name]

    res = joint(tree, aln, mult, model, full_length)
    set_lengths(res)
    n = 0
    while n < max_iter:
        n += 1
        if prune_short:
            prune_short_branches(tree, cseq_of(res["cseq"]), mult, model, one_mutation)
        res = joint(tree, aln, mult, model, full_length, prev_cseq=res["cseq"])
        if res["N_diff"] < 1:
            break
        set_lengths(res)
    return res, float((res["sequence_LH"] * mult).sum())


# --------------------------------------------------------------- compression
def seq2array(seq, fill_overhangs=False, ambiguous="N", convert_upper=True):
    """seq_utils.py:152-204 for word length 1."""
    s = seq.upper() if convert_upper else seq
    arr = np.array(list(s))
    if fill_overhangs:
        gaps = np.where(arr != "-")[0]
        if len(gaps):
            arr[: gaps[0]] = ambiguous
            arr[gaps[-1] + 1:] = ambiguous
        else:
            arr[:] = ambiguous
    return arr


def compress_alignment(names, arrays, ambiguous):
    """SequenceData.make_compressed_alignment (sequence_data.py:325-464) for a
    dense alignment: per-column loop with string pattern keys.  Returns
    (compressed dict name -> chars, multiplicity, full_to_compressed,
    compressed_to_full)."""
    aln_t = np.array([arrays[k] for k in names]).T
    patterns = {}
    columns = []
    for pi in range(aln_t.shape[0]):
        pattern = np.copy(aln_t[pi])
        letters = list(np.unique(pattern))
        if len(letters) == 2 and ambiguous in letters:
            other = [c for c in letters if c != ambiguous][0]
            pattern[pattern == ambiguous] = other
            letters = [other]
        key = "".join(pattern.astype("U"))
        if len(letters) > 1:
            key += "_%d" % pi
        if key not in patterns:
            patterns[key] = (len(columns), [pi])
            columns.append(pattern)
        else:
            patterns[key][1].append(pi)
    mult = np.zeros(len(patterns))
    for p, pos in patterns.values():
        mult[p] = len(pos)
    comp = np.array(columns).T
    compressed = {k: comp[i] for i, k in enumerate(names)}
    f2c = np.zeros(aln_t.shape[0], dtype=int)
    for p, pos in patterns.values():
        f2c[np.array(pos)] = p
    c2f = {val[0]: np.array(val[1], dtype=int) for val in patterns.values()}
    return compressed, mult, f2c, c2f
