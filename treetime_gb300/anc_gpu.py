"""``GPUAncMixin``: the reconstruction and branch-length methods of TreeAnc
implemented on the GPU.

The mixin replaces exactly the hot-path methods of treetime/treeanc.py:
``_ml_anc_marginal`` (:762), ``_ml_anc_joint`` (:934), ``_fitch_anc`` (:575),
``optimize_branch_lengths_joint`` (:1176), ``optimal_branch_length`` (:1244),
``optimal_marginal_branch_length`` (:1272), ``optimize_tree_marginal``
(:1297), ``prune_short_branches`` (:1475), ``get_branch_mutation_matrix``
(:1085), ``infer_gtr`` (:1500) and ``infer_gtr_iterative`` (:1633), and adds
``branch_length_grids`` (the values of BranchLenInterpolator,
treetime/branch_len_interpolator.py:36-125).  It reads only the state
TreeTime's own classes keep (``tree``, ``data``, ``gtr``, ``rng``,
``sequence_reconstruction``, ``reconstructed_tip_sequences``,
``use_mutation_length``, ``ignore_gaps``, ``logger``), so it composes with
``treetime_gb300.TreeAnc`` and, placed first in the MRO, with TreeTime's own
classes::

    class TreeTimeGPU(GPUAncMixin, treetime.TreeTime): pass

Nodes of ``treetime_gb300.tree.Clade`` receive their per-node arrays lazily;
other clade objects (Bio.Phylo) receive them as attributes right away.
"""

import ctypes as C
import itertools
import operator

import numpy as np

from . import config as ttconf
from . import engine
from .alphabets import chars_to_codes, profile_lut
from .errors import MissingDataError
from .tree import LAZY_ATTRS, Clade, assign_lengths, length_epoch, topology_epoch


def _dist2root(layout, lengths):
    """dist2root of every node from the root's 0 and each node's length, parents
    before children (internal nodes by decreasing height, then the tips): the
    additions of TreeTime's _calc_dist2root (treetime/treeanc.py:499-510), in
    numpy, one height level at a time."""
    steps = getattr(layout, "_d2r_steps", None)
    if steps is None:  # (nodes, their parents) per level from the top, then the tips; per layout
        par = np.asarray(layout.parent)
        lev = layout.level_off
        steps = []
        for h in range(layout.n_levels - 1, -1, -1):
            ks = np.arange(lev[h], lev[h + 1])
            ks = ks[par[ks] >= 0]
            steps.append((ks, par[ks]))
        tips = np.arange(layout.n_int, layout.n_nodes)
        steps.append((tips, par[tips]))
        layout._d2r_steps = steps
    d = np.zeros(layout.n_nodes)
    for ks, pk in steps:
        d[ks] = d[pk] + lengths[ks]
    return d


def _set_dist2root(layout, lengths):
    """_dist2root stored on the nodes."""
    for node, v in zip(layout.nodes, _dist2root(layout, lengths).tolist()):
        node.dist2root = v


_CLADES = operator.attrgetter("clades")
_END = object()  # closes the list of children, so that a longer or shorter list differs


def _children(nodes):
    """Every child of every node, in order, then _END (C-level iteration): the
    same objects in the same order mean an unchanged topology below the same
    root."""
    return list(itertools.chain(itertools.chain.from_iterable(map(_CLADES, nodes)), (_END,)))


def _same_children(nodes, ref):
    """The nodes' children are the objects of ``ref`` (from _children), in order
    (compared by identity, without building a list)."""
    return all(map(operator.is_, itertools.chain(itertools.chain.from_iterable(map(_CLADES, nodes)), (_END,)), ref))


def _masks(nodes):
    return list(map(getattr, nodes, itertools.repeat("mask"), itertools.repeat(None)))


def _same_masks(nodes, ref):
    return all(map(operator.is_, map(getattr, nodes, itertools.repeat("mask"), itertools.repeat(None)), ref))


class ResultHolder:
    """The results a session's clades show (their ``_anc_src``): installing a
    reconstruction replaces the holder's source, one assignment for the whole
    tree.  Values assigned to a clade's result attributes (tree._Result)
    override the source until the next installation."""

    def __init__(self):
        self.src = None
        self._overridden = []

    def fetch(self, name, node):
        return None if self.src is None else self.src.fetch(name, node)

    def overridden(self, node):
        self._overridden.append(node)

    def install(self, src):
        for n in self._overridden:
            ov = n.__dict__.get("_anc_override")
            if ov:
                ov.clear()
        self._overridden.clear()
        self.src = src


def pair_counts(seq_p, seq_ch, mult, q, gap_index, ignore_gaps):
    """[q, q] multiplicity-weighted counts of (parent state, child state) over
    the patterns of two state-index sequences, positions with a gap on either
    side left out when `ignore_gaps` (GTR.state_pair, treetime/gtr.py:631-712,
    before its cast to integers)."""
    w = np.asarray(mult, dtype=float)
    a = np.asarray(seq_p, dtype=np.int64)
    b = np.asarray(seq_ch, dtype=np.int64)
    if ignore_gaps and gap_index is not None:
        w = np.where((a == gap_index) | (b == gap_index), 0.0, w)
    return np.bincount(a * q + b, weights=w, minlength=q * q).reshape(q, q)


_PINNED = {}


def _pinned_copy(t):
    """Host copy of a device tensor through a reused page-locked buffer (one
    asynchronous copy on the current stream, then a wait for it); the array
    returned is the caller's own."""
    torch = engine.torch()
    n = t.numel() * t.element_size()
    buf = _PINNED.get(t.dtype)
    if buf is None or buf.numel() * buf.element_size() < n:
        buf = torch.empty(max(n // t.element_size(), 1), dtype=t.dtype, pin_memory=True)
        _PINNED[t.dtype] = buf
    view = buf[:t.numel()]
    view.copy_(t.reshape(-1), non_blocking=True)
    torch.cuda.current_stream(t.device).synchronize()
    return view.numpy().copy()


def _pinned_pair(sess, a, b):
    """Host copies of two small device tensors through page-locked buffers of
    the session: two asynchronous copies, one wait."""
    torch = engine.torch()
    if not a.is_cuda:  # host tensors (stand-ins of the device pieces in host-logic tests)
        return a.numpy().copy(), b.numpy().copy()
    bufs = sess.setdefault("pinned_small", {})
    outs = []
    for key, x in (("a", a), ("b", b)):
        buf = bufs.get((key, x.dtype))
        if buf is None or buf.numel() < x.numel():
            buf = torch.empty(max(x.numel(), 1), dtype=x.dtype, pin_memory=True)
            bufs[(key, x.dtype)] = buf
        view = buf[:x.numel()]
        view.copy_(x.reshape(-1), non_blocking=True)
        outs.append(view)
    torch.cuda.current_stream(a.device).synchronize()
    return tuple(v.numpy().copy().reshape(x.shape) for v, x in zip(outs, (a, b)))


def _pinned_results(sess, P):
    """The session's page-locked result buffers (states of every node, site
    and tree log-likelihoods, changed-site count, status word), made once at
    their largest size: the session's CUDA graphs copy into them, so they are
    never replaced."""
    pb = sess.get("pinned")
    if pb is None:
        torch = engine.torch()
        n = sess["layout"].n_nodes * P
        pb = (torch.empty(max(n, 1), dtype=torch.uint8, pin_memory=True),
              torch.empty(P + 1, dtype=torch.float64, pin_memory=True),
              torch.empty(1, dtype=torch.int64, pin_memory=True),
              torch.empty(1, dtype=torch.int32, pin_memory=True))
        sess["pinned"] = pb
    return pb


def _copy_results(sess, out, rows, P, site_key="site_lh", tree_key="tree_lh", n_diff=True):
    """Asynchronous copies of a reconstruction's host results into the
    session's page-locked buffers, on the current stream (also inside a CUDA
    graph capture)."""
    torch = engine.torch()
    st, sc, nd, stat = _pinned_results(sess, P)
    nb = rows * P
    stat.copy_(sess["bufs"].get("status", (1,), torch.int32), non_blocking=True)
    st[:nb].copy_(out["states"].view(-1)[:nb], non_blocking=True)
    sc[:P].copy_(out[site_key][:P], non_blocking=True)
    sc[P:P + 1].copy_(out[tree_key][:1], non_blocking=True)
    if n_diff:
        nd.copy_(out["n_diff"][:1], non_blocking=True)


def _host_results(sess, out, rows, P, site_key="site_lh", tree_key="tree_lh", n_diff=True, copied=False):
    """The results every reconstruction hands to the host -- the states of the
    reconstructed rows, the site and tree log-likelihoods and the changed-site
    count -- through page-locked buffers of the session, as asynchronous copies
    on the current stream (already queued when `copied`: a session graph
    holds them) followed by one wait; the kernels' status word comes with them
    (the passes are launched without a wait of their own) and is checked
    before anything is returned.  The states array returned is a view of the
    session's buffer: valid until the session's next reconstruction (the
    results installed on the nodes read it only until then)."""
    torch = engine.torch()
    if not copied:
        _copy_results(sess, out, rows, P, site_key, tree_key, n_diff)
    st, sc, nd, stat = _pinned_results(sess, P)
    torch.cuda.current_stream(out["states"].device).synchronize()
    s = int(stat.numpy()[0])
    if s:
        engine.check(s, "kernel status")
    scn = sc.numpy()
    nb = rows * P
    return (st.numpy()[:nb].reshape(rows, P), scn[:P].copy(), float(scn[P]),
            int(nd.numpy()[0]) if n_diff else 0)


class ResultStore:
    """Host view of one reconstruction's device results; node attributes are
    built from it on first access."""

    def __init__(self, tt, layout, kind, out, precision, reconstruct_tips, states=None):
        self.tt = tt
        self.layout = layout
        self.kind = kind
        self.out = out
        self.precision = precision
        self.reconstruct_tips = reconstruct_tips
        self.P = tt.data.compressed_length
        self.q = tt.gtr.n_states
        # the reconstructed rows: internal nodes, and the tips when their states were reconstructed
        rows = layout.n_nodes if reconstruct_tips else layout.n_int
        if states is None:
            states = _pinned_copy(out["states"].view(-1)[: rows * self.P]).reshape(rows, self.P)
        self.states = states
        self._host = {}
        self._cache = {}

    def _fetch_buf(self, key):
        if key not in self._host:
            if key in ("outgroup", "tip_outgroup") and self.out.get("_outgroups") is not None:
                self.out["_outgroups"]()  # rows formed on request (engine.outgroups)
            buf = self.out.get(key)
            self._host[key] = None if buf is None else buf.cpu().numpy()
        return self._host[key]

    def _rows(self, key, j):
        buf = self._fetch_buf(key)
        if buf is None:
            return None
        return buf[j * self.P:(j + 1) * self.P, :self.q].astype(np.float64)

    def fetch(self, name, node):
        key = (name, id(node))
        hit = self._cache.get(key)
        if hit is None:
            hit = self._fetch(name, node)
            if hit is not None:
                self._cache[key] = hit
        return hit

    def _fetch(self, name, node):
        L = self.layout
        k = L.local.get(id(node))
        if k is None:
            return None
        is_tip = k >= L.n_int
        if name == "_cseq":
            if is_tip and not self.reconstruct_tips:
                return None
            if self.kind == "parsimony":  # characters, possibly outside the alphabet
                chars = self._fetch_buf("chars")
                return chars[k * self.P:(k + 1) * self.P].view("S1").astype("U1")
            return self.tt.gtr.alphabet[self.states[k]]
        if self.kind != "marginal":
            return None
        if name == "marginal_profile":
            return self._rows("tip_posterior", k - L.n_int) if is_tip else self._rows("posterior", k)
        if name == "marginal_subtree_LH":
            if is_tip:
                return self.tt._tip_profile(node)
            x = self._rows("partial", k)
            if self.precision == "f32":  # FP32 partials are power-of-two scaled: normalise in FP64
                x = x.astype(np.float64)
                x = x / x.sum(axis=1, keepdims=True)
            return x
        if name == "marginal_outgroup_LH":
            if k == L.n_int - 1:
                return self.tt._root_outgroup()
            return self._rows("tip_outgroup", k - L.n_int) if is_tip else self._rows("outgroup", k)
        return None


class BranchStateStore:
    """``branch_state`` dictionaries from the pair histograms (a device tensor
    of this store's own, copied to the host on the first read, or a host
    array)."""

    def __init__(self, layout, hist):
        self.layout = layout
        self._hist = hist
        self._host = None

    @property
    def hist(self):
        if self._host is None:
            h = self._hist
            self._host = h.cpu().numpy() if hasattr(h, "cpu") else np.asarray(h)
        return self._host

    def fetch(self, name, node):
        if name != "branch_state":
            return None
        k = self.layout.local.get(id(node))
        if k is None or getattr(node, "up", None) is None:
            return None
        h = self.hist[k]
        idx = np.argwhere(h != 0)
        return {"pair": idx.astype(int), "multiplicity": h[idx[:, 0], idx[:, 1]].astype(int)}


class _ChainedSource:
    def __init__(self, *srcs):
        self.srcs = [s for s in srcs if s is not None]

    def fetch(self, name, node):
        for s in self.srcs:
            v = s.fetch(name, node)
            if v is not None:
                return v
        return None


class GPUAncMixin:
    """GPU implementations of TreeAnc's reconstruction and branch-length methods."""

    # ----------------------------------------------------------- device session
    def _gpu_precision(self):
        return getattr(self, "precision", "f64")

    def _aln_index(self):
        """(name -> row, compressed byte matrix) of the alignment."""
        d = self.data
        if hasattr(d, "compressed_codes") and hasattr(d, "name_to_row"):
            return d.name_to_row, d.compressed_codes
        key = (id(d), d.compressed_length, id(d.compressed_alignment))
        cache = getattr(self, "_aln_index_cache", None)
        if cache is None or cache[0] != key:
            names = list(d.compressed_alignment.keys())
            codes = np.stack([chars_to_codes(d.compressed_alignment[k]) for k in names])
            cache = (key, {k: i for i, k in enumerate(names)}, codes)
            self._aln_index_cache = cache
        return cache[1], cache[2]

    def _get_session(self):
        """Device-resident schedule and inputs of the current tree, rebuilt when
        the topology (any node's list of children), alignment, model or masks
        change; branch lengths are refreshed on every call.  The checks are
        C-level iterations over the session's nodes."""
        s = getattr(self, "_session", None)
        gtr_key = engine.model_key(self.gtr)
        if s is not None and s["root"] is self.tree.root and s["data"] is self.data and s["gtr_key"] == gtr_key:
            nodes = s["layout"].nodes
            # a tree of this package's clades that nothing has changed since (tree.topology_epoch)
            # needs no walk; otherwise every child and mask is compared by identity
            epoch = topology_epoch()
            if (s["own"] and epoch == s["epoch"]) or (_same_children(nodes, s["children"]) and
                                                       _same_masks(nodes, s["masks"])):
                s["epoch"] = epoch
                self._refresh_lengths(s)
                return s
        engine.check_alphabet(self.gtr.n_states, self.gtr.is_site_specific)
        device = getattr(self, "device", None)
        layout = engine.TreeLayout(self.tree.root)
        name_to_row, codes = self._aln_index()
        tip_row = np.full(layout.n_tip, -1, dtype=np.int32)
        for j, n in enumerate(layout.nodes[layout.n_int:]):
            r = name_to_row.get(n.name)
            if r is not None:
                tip_row[j] = r
        masks, mask_ids = {}, {}
        for k, n in enumerate(layout.nodes):
            m = getattr(n, "mask", None)
            if m is not None:
                masks[k] = np.asarray(m, dtype=np.float64)
                mask_ids[k] = id(m)
        bl_key = self._lengths_key()
        bl = engine.branch_lengths(layout, self.data.full_length, self.use_mutation_length)
        engine.check_exp(self.gtr, bl)
        ti = engine.TreeInput(layout, codes, tip_row, self.data.multiplicity(), bl, masks=masks)
        forest = engine.Forest([ti], self.gtr.n_states, device=device,
                               threads=getattr(self, "threads", None),
                               warps_per_block=getattr(self, "warps_per_block", None),
                               ctas_per_sm=getattr(self, "ctas_per_sm", None) or 1,
                               range_patterns=getattr(self, "range_patterns", None))
        model = None if self.gtr.is_site_specific else engine.model_for(self.gtr, device)
        holder = ResultHolder()
        foreign = []
        rm = LAZY_ATTRS + ("_anc_src", "_anc_override", "joint_Lx", "joint_Cx", "seq_idx", "marginal_log_Lx",
                           "marginal_subtree_LH_prefactor")
        for n in layout.nodes:
            d = n.__dict__
            for a in rm:
                d.pop(a, None)
            if isinstance(n, Clade):
                d["_anc_src"] = holder
            else:
                foreign.append(n)
        s = dict(layout=layout, forest=forest, model=model, bufs=engine.Buffers(forest), mask_ids=mask_ids,
                 root=self.tree.root, data=self.data, gtr_key=gtr_key, n_nodes=layout.n_nodes,
                 children=_children(layout.nodes), masks=_masks(layout.nodes), holder=holder,
                 foreign=foreign, own=not foreign, epoch=topology_epoch(), bl_key=bl_key,
                 dicts=None if foreign else [n.__dict__ for n in layout.nodes])
        self._session = s
        return s

    def _lengths_key(self):
        return (length_epoch(), self.data.full_length, bool(self.use_mutation_length))

    def _refresh_lengths(self, s):
        """Branch lengths to the device, unless the session's copy is current: a
        tree of this package's clades none of whose branch lengths was assigned
        since the copy (tree.length_epoch), for the same alignment length (the
        floor 1e-3 / L) and length attribute.  Otherwise every node is read."""
        key = self._lengths_key()
        if s["own"] and not key[2] and s["bl_key"] == key:
            return
        bl = engine.branch_lengths(s["layout"], self.data.full_length, self.use_mutation_length)
        engine.check_exp(self.gtr, bl)
        s["forest"].set_branch_lengths([bl])
        s["bl_key"] = key

    def _tip_profile(self, node):
        name_to_row, codes = self._aln_index()
        r = name_to_row.get(node.name)
        if r is None:
            return np.ones((self.data.compressed_length, self.gtr.n_states))
        return profile_lut(self.gtr.profile_map, self.gtr.n_states)[codes[r]]

    def _root_outgroup(self):
        Pi = np.asarray(self.gtr.Pi)
        L = self.data.compressed_length
        return np.repeat([Pi], L, axis=0) if Pi.ndim == 1 else np.copy(Pi.T)

    def _seed_tip_states(self, sess):
        """Before the first reconstruction that includes tips, tip rows of the
        state buffer hold the alignment's states (255 for characters that are not
        states), so changed-site counts compare against the alignment as TreeTime
        does."""
        layout = sess["layout"]
        P = self.data.compressed_length
        name_to_row, codes = self._aln_index()
        strict = np.full(256, 255, np.uint8)
        for i, c in enumerate(self.gtr.alphabet):
            strict[ord(str(c))] = i
        tip = np.full((layout.n_tip, P), 255, dtype=np.uint8)
        for j, n in enumerate(layout.nodes[layout.n_int:]):
            r = name_to_row.get(n.name)
            if r is not None:
                tip[j] = strict[codes[r]]
        states = sess["bufs"].get("states", (sess["forest"].state_rows,), engine.torch().uint8)
        states[layout.n_int * P:].copy_(engine.torch().from_numpy(tip.reshape(-1)))

    def _clear_results(self, layout):
        """Results of an earlier reconstruction leave with the next one: the
        session's clades ask its result holder (replaced by _install); other
        clade objects carry plain attributes, removed here."""
        sess = self._session
        rm = LAZY_ATTRS + ("joint_Lx", "joint_Cx", "seq_idx", "marginal_log_Lx", "marginal_subtree_LH_prefactor")
        for n in sess["foreign"]:
            d = n.__dict__
            for a in rm:
                d.pop(a, None)

    def _install(self, src, layout):
        sess = self._session
        sess["holder"].install(src)
        for n in sess["foreign"]:  # foreign clade objects: materialise eagerly
            for a in LAZY_ATTRS:
                v = src.fetch(a, n)
                if v is not None:
                    setattr(n, a, v)

    def _pass(self, sess, fn, key, rows, *args, **kw):
        """One pass of the session launched without a wait, returning (device outputs, whether
        the host results are already queued for copying): the first call with a set of options
        runs it directly, the second captures it as a CUDA graph (engine.CapturedCall) together
        with the copies of its host results into the session's page-locked buffers, later ones
        replay the graph -- the same kernels and copies on the same buffers with one host call
        instead of a dozen launches.  The graphs live with the session (a new topology, alignment
        or model starts without them); branch lengths and tip codes are read at replay."""
        graphs = sess.setdefault("graphs", {})
        g = graphs.get(key)
        if g is None:
            graphs[key] = 1
            return fn(*args, sync=False, **kw), False
        if g == 1:
            P = self.data.compressed_length
            _pinned_results(sess, P)  # page-locked memory is allocated outside the capture
            g = graphs[key] = engine.CapturedCall(fn, *args, after=lambda out: _copy_results(sess, out, rows, P),
                                                  **kw)
        return g.replay(), True

    def _root_draws(self, sample_from_profile):
        """The root's uniform draws (sample_from_profile 'root' or True), one
        rng.random(L) as TreeTime's prof2seq (treetime/seq_utils.py:265-269)."""
        if sample_from_profile == "root" or sample_from_profile is True:
            return self.rng.random(size=self.data.compressed_length)
        return None

    def _node_draws(self, layout, reconstruct_tip_states):
        """sample_from_profile=True: one rng.random(L) per node whose state is
        drawn, in preorder after the root's (treetime/treeanc.py:880-932): the
        internal nodes, and the tips when their states are reconstructed; laid
        out by node id like the states (the other rows are not read)."""
        P = self.data.compressed_length
        out = np.zeros(layout.n_nodes * P)
        for n in self.tree.find_clades(order="preorder"):
            if n.up is None or (not n.clades and not reconstruct_tip_states):
                continue
            k = layout.local[id(n)]
            out[k * P:(k + 1) * P] = self.rng.random(size=P)
        return out

    # --------------------------------------------------------- reconstruction
    def _ml_anc_marginal(self, sample_from_profile=False, reconstruct_tip_states=False, debug=False,
                         keep_outgroup=True, **kwargs):
        """Marginal reconstruction in one device pass (treetime/treeanc.py:762-932)."""
        self.logger("TreeAnc._ml_anc_marginal: type of reconstruction: Marginal (GPU)", 2)
        sess = self._get_session()
        layout = sess["layout"]
        count_diff = bool(self.sequence_reconstruction)
        if reconstruct_tip_states and count_diff and not self.reconstructed_tip_sequences:
            self._seed_tip_states(sess)
        draws = self._root_draws(sample_from_profile)
        node_draws = self._node_draws(layout, reconstruct_tip_states) if sample_from_profile is True else None
        prec = self._gpu_precision()
        kw = dict(precision=prec, reconstruct_tips=reconstruct_tip_states, keep_outgroup=keep_outgroup,
                  tip_outgroup=keep_outgroup, count_diff=count_diff, root_uniform=draws, node_uniform=node_draws)
        rows = layout.n_nodes if reconstruct_tip_states else layout.n_int
        copied = False
        if prec == "f32" and not self.gtr.is_site_specific and self.gtr.n_states <= 5:
            # the pass without its outgroup rows (formed when first asked for, from the branch
            # lengths it used) and with the changed-site count by a compare kernel: the same
            # results, without the pre-order's tip level and the outgroup stores
            snap = sess.setdefault("snap", {})
            lkw = dict(reconstruct_tips=reconstruct_tip_states, count_diff=count_diff, root_uniform=draws,
                       node_uniform=node_draws)
            if draws is None and node_draws is None:
                out, copied = self._pass(sess, engine.marginal_lean, ("lean",) + tuple(sorted(lkw.items())), rows,
                                         sess["forest"], sess["model"], sess["bufs"], snap, **lkw)
            else:
                out = engine.marginal_lean(sess["forest"], sess["model"], sess["bufs"], snap, sync=False, **lkw)
            out = dict(out)  # this reconstruction's view: its outgroup rows are not formed yet
            out["outgroup"] = out["tip_outgroup"] = None
            if keep_outgroup:
                scratch = sess.get("og_scratch")
                if scratch is None:
                    scratch = sess["og_scratch"] = engine.Buffers(sess["forest"])
                f, m, b = sess["forest"], sess["model"], sess["bufs"]
                out["_outgroups"] = lambda o=out: engine.outgroups(f, m, b, o, snap, scratch)
        elif self.gtr.is_site_specific:
            out = engine.marginal_site_specific(sess["forest"], self.gtr, sess["bufs"], sync=False, **kw)
        elif draws is None and node_draws is None:
            out, copied = self._pass(sess, engine.marginal, ("marginal",) + tuple(sorted(kw.items())), rows,
                                     sess["forest"], sess["model"], sess["bufs"], **kw)
        else:
            out = engine.marginal(sess["forest"], sess["model"], sess["bufs"], sync=False, **kw)
        self._clear_results(layout)
        P = self.data.compressed_length
        n_recon = layout.n_int - 1 + (layout.n_tip if reconstruct_tip_states else 0)
        states, site_lh, total, nd = _host_results(sess, out, rows, P, copied=copied)
        N_diff = nd if count_diff else P * n_recon
        self._install(ResultStore(self, layout, "marginal", out, prec, reconstruct_tip_states, states=states),
                      layout)
        self.tree.sequence_LH = site_lh
        self.tree.total_sequence_LH = total
        self.tree.sequence_marginal_LH = self.tree.total_sequence_LH
        self.reconstructed_tip_sequences = reconstruct_tip_states
        self.sequence_reconstruction = "marginal"
        self._last = ("marginal", out)
        return N_diff

    def _ml_anc_joint(self, sample_from_profile=False, reconstruct_tip_states=False, debug=False, **kwargs):
        """Joint reconstruction in one device pass (treetime/treeanc.py:934-1080)."""
        self.logger("TreeAnc._ml_anc_joint: type of reconstruction: Joint (GPU)", 2)
        sess = self._get_session()
        layout = sess["layout"]
        count_diff = bool(self.sequence_reconstruction)
        if reconstruct_tip_states and count_diff and not self.reconstructed_tip_sequences:
            self._seed_tip_states(sess)
        draws = self._root_draws(sample_from_profile)
        rows = layout.n_nodes if reconstruct_tip_states else layout.n_int
        copied = False
        if self.gtr.is_site_specific:
            out = engine.joint_site_specific(sess["forest"], self.gtr, sess["bufs"],
                                             reconstruct_tips=reconstruct_tip_states, count_diff=count_diff,
                                             root_uniform=draws, sync=False)
        elif draws is None:
            out, copied = self._pass(sess, engine.joint, ("joint", reconstruct_tip_states, count_diff), rows,
                                     sess["forest"], sess["model"], sess["bufs"],
                                     reconstruct_tips=reconstruct_tip_states, count_diff=count_diff)
        else:
            out = engine.joint(sess["forest"], sess["model"], sess["bufs"], reconstruct_tips=reconstruct_tip_states,
                               count_diff=count_diff, root_uniform=draws, sync=False)
        self._clear_results(layout)
        P = self.data.compressed_length
        n_recon = layout.n_int - 1 + (layout.n_tip if reconstruct_tip_states else 0)
        states, site_lh, total, nd = _host_results(sess, out, rows, P, copied=copied)
        N_diff = nd if count_diff else P * n_recon
        self._install(ResultStore(self, layout, "joint", out, "f64", reconstruct_tip_states, states=states), layout)
        self.tree.sequence_LH = site_lh
        self.tree.sequence_joint_LH = total
        self.reconstructed_tip_sequences = reconstruct_tip_states
        self.sequence_reconstruction = "joint"
        self._last = ("joint", out)
        return N_diff

    def _previous_chars(self, sess):
        """Characters of the last reconstruction in the state layout (device),
        or None when there is none."""
        t = engine.torch()
        last = getattr(self, "_last", None)
        if not self.sequence_reconstruction or last is None:
            return None
        if last[0] == "parsimony":
            return last[1]["chars"].clone()
        states = sess["bufs"].cache.get(("states", t.uint8))
        if states is None:
            return None
        alpha = np.zeros(256, dtype=np.uint8)
        alpha[:len(self.gtr.alphabet)] = np.frombuffer("".join(self.gtr.alphabet.tolist()).encode(), np.uint8)
        return engine._to_dev(alpha, states.device)[states.long()]

    def _fitch_anc(self, **kwargs):
        """Fitch parsimony (treetime/treeanc.py:575-643) on the GPU: the lists
        of all internal nodes in one pass up the tree, the root's characters on
        the host (a random entry of a longer list from TreeTime's generator, in
        position order), one pass down."""
        t = engine.torch()
        lib = engine._lib.load()
        sess = self._get_session()
        layout, forest, bufs = sess["layout"], sess["forest"], sess["bufs"]
        P = self.data.compressed_length
        tip_chars = None
        if self.reconstructed_tip_sequences:
            tip_chars = self._previous_chars(sess)
        else:
            missing = self._missing_tip(sess)
            if missing is not False:
                raise MissingDataError("TreeAnc._fitch_anc: terminal node alignments required; sequence is "
                                       "missing for leaf: '%s'." % missing)
        prev = self._previous_chars(sess)
        lists = bufs.get("fitch_lists", (forest.prof_rows, 16), t.uint8)
        status = bufs.get("status", (1,), t.int32)
        status.zero_()
        engine.check(lib.tt_fitch_up(C.byref(forest.struct), engine._p(lists), engine._p(tip_chars),
                                     engine._p(status), engine._stream()), "tt_fitch_up")
        engine._check_status(status)
        self.logger("TreeAnc._fitch_anc: Walking up the tree, creating the Fitch profiles", 2)
        root = lists[(layout.n_int - 1) * P:layout.n_int * P].cpu().numpy()
        lens = root[:, 15].astype(np.int64)
        root_chars = root[:, 0].copy()
        amb = np.flatnonzero(lens > 1)
        if amb.size and 4 < getattr(self, "verbose", 5):  # messages formed only when they are printed
            for i in amb:
                choices = root[i, :lens[i]].tobytes().decode("latin-1")
                self.logger("Ambiguous state of the root sequence in the position %d: %s, choosing %s"
                            % (i, str(list(choices)), choices[0]), 4)
        if amb.size:
            # one draw per ambiguous position in position order (treetime/treeanc.py:615-617): a
            # vector of bounds gives the scalar calls' sequence and leaves the generator in the
            # same state
            root_chars[amb] = root[amb, self.rng.integers(lens[amb])]
        self.logger("TreeAnc._fitch_anc: Walking down the self.tree, generating sequences from the Fitch profiles.", 2)
        chars = bufs.get("fitch_chars", (forest.state_rows,), t.uint8)
        states = bufs.get("states", (forest.state_rows,), t.uint8)
        if tip_chars is not None:
            chars[layout.n_int * P:].copy_(tip_chars[layout.n_int * P:])
        n_diff = t.zeros(1, dtype=t.int64, device=forest.device)
        d_root = engine._to_dev(root_chars, forest.device)
        cs = engine._to_dev(engine.char_state_table(self.gtr, strict=True), forest.device)
        engine.check(lib.tt_fitch_down(C.byref(forest.struct), engine._p(lists), engine._p(d_root), engine._p(chars),
                                       engine._p(states), engine._p(cs), engine._p(prev), engine._p(n_diff),
                                       engine._stream()), "tt_fitch_down")
        N_diff = int(n_diff.item()) if prev is not None else (layout.n_int - 1) * P
        self._clear_results(layout)
        out = {"states": states, "chars": chars}
        self._install(ResultStore(self, layout, "parsimony", out, "f64", self.reconstructed_tip_sequences), layout)
        self.sequence_reconstruction = "parsimony"
        self._last = ("parsimony", out)
        self.logger("Done ancestral state reconstruction", 3)
        return N_diff

    def _missing_tip(self, sess):
        """The name of a tip without an alignment row, or False.  The session's tips and their
        rows are fixed when it is built, so the tips are looked through once per session."""
        missing = sess.get("tip_missing")
        if missing is None:
            layout = sess["layout"]
            name_to_row, _ = self._aln_index()
            missing = sess["tip_missing"] = next(
                (n.name for n in layout.nodes[layout.n_int:] if n.name not in name_to_row), False)
        return missing

    # --------------------------------------------------------- branch lengths
    def _pair_histograms(self, ignore_gaps=None):
        """(session, [n_nodes, q, q] device histograms of (parent, child) states
        per branch), gaps excluded when `ignore_gaps` (default: the instance's
        setting)."""
        sess = self._get_session()
        layout = sess["layout"]
        if not self.reconstructed_tip_sequences:
            missing = self._missing_tip(sess)
            if missing is not False:
                raise MissingDataError(
                    "TreeAnc.optimal_branch_length: terminal node alignments required; sequence is missing for "
                    "leaf: '%s'. Missing terminal sequences can be inferred from sister nodes by rerunning with "
                    "`reconstruct_tip_states=True` or `--reconstruct-tip-states`" % missing)
        ig = self.ignore_gaps if ignore_gaps is None else ignore_gaps
        cs = sess.get("char_state")  # the alphabet's byte -> state table (the model is the session's)
        if cs is None:
            cs = sess["char_state"] = engine._to_dev(engine.char_state_table(self.gtr), sess["forest"].device)
        hist, _ = engine.state_pairs(sess["forest"], sess["bufs"], cs, self.gtr.gap_index, ig,
                                     self.reconstructed_tip_sequences)
        return sess, hist

    def optimize_branch_lengths_joint(self, **kwargs):
        """All branches in one device pass: pair histograms, then Brent per
        branch (treetime/treeanc.py:1176-1242)."""
        self.logger("TreeAnc.optimize_branch_length: running branch length optimization using jointML ancestral "
                    "sequences", 1)
        if self.tree is None or self.data is None or self.data.aln is None:
            raise MissingDataError("TreeAnc.optimize_branch_length: ERROR, alignment or tree are missing.")
        if not self.sequence_reconstruction:
            raise ValueError("Ancestral sequences are not yet inferred")
        store_old = kwargs.get("store_old", False)
        sess, hist = self._pair_histograms()
        layout = sess["layout"]
        counts = engine.torch().trunc(hist)  # TreeTime casts pair counts to int
        t, info = engine.optimal_t_pairs(self.gtr.n_states, counts, sess["model"], tol=1e-10)
        t, info = _pinned_pair(sess, t, info)
        root_k = layout.n_int - 1
        failed = info == -1
        failed[root_k] = False
        if failed.any():
            engine.check(engine._lib.TT_ERR_BRACKET, "optimize_branch_lengths_joint")
        lengths = np.maximum(0.0, t)
        lengths[root_k] = 0.0
        max_bl = float(lengths.max()) if len(lengths) else 0.0
        if (lengths > 0.9 * ttconf.MAX_BRANCH_LENGTH).any():
            self.logger("WARNING: GTR.optimal_t_compressed -- The branch length seems to be very long!", 4, warn=True)
        rest = layout.nodes[:root_k] + layout.nodes[root_k + 1:]  # every node but the root
        vals = lengths[:root_k].tolist() + lengths[root_k + 1:].tolist()
        if store_old:
            for node in rest:
                node._old_length = node.branch_length
        from .treeanc import TreeAnc as _OwnTreeAnc  # (treeanc imports this module)
        # with TreeAnc's own _prepare_nodes, of what it re-derives only the distances to the root
        # change (the topology is the session's, checked when this call began)
        own_prepare = type(self)._prepare_nodes is _OwnTreeAnc._prepare_nodes
        dicts = sess.get("dicts") if sess.get("own") else None
        d2r = None
        if dicts is not None and not self.use_mutation_length:
            # the session's clades take the lengths (and distances to the root) in one loop with
            # one bump of the change counter, and the device copy is made here from the same
            # numbers (the root keeps its length)
            if own_prepare:
                d2r = _dist2root(layout, lengths).tolist()
                dicts[root_k]["dist2root"] = 0.0
            assign_lengths(dicts[:root_k] + dicts[root_k + 1:], vals,
                           None if d2r is None else d2r[:root_k] + d2r[root_k + 1:])
            bl = lengths.astype(np.float64)
            r = layout.nodes[root_k].branch_length
            bl[root_k] = np.nan if r is None else r
            bl = engine.length_floor(bl, self.data.full_length)
            try:
                engine.check_exp(self.gtr, bl)
            except ValueError:
                sess["bl_key"] = None  # the next call reads the lengths again and raises there
            else:
                sess["forest"].set_branch_lengths([bl])
                sess["bl_key"] = self._lengths_key()
        else:
            for node, new_len in zip(rest, vals):
                node.branch_length = new_len
                node.mutation_length = new_len
        bstore = BranchStateStore(layout, counts)
        holder = sess.get("holder")
        if holder is not None:
            holder.install(_ChainedSource(holder.src, bstore) if holder.src is not None else bstore)
        for n in (sess.get("foreign", ()) if holder is not None else layout.nodes):
            v = bstore.fetch("branch_state", n)
            if v is not None:
                n.branch_state = v
        if max_bl > 0.15:
            self.logger("TreeAnc.optimize_branch_lengths_joint: THIS TREE HAS LONG BRANCHES."
                        " \n\t ****TreeTime's JOINT IS NOT DESIGNED TO OPTIMIZE LONG BRANCHES."
                        " \n\t ****PLEASE OPTIMIZE BRANCHES USING: "
                        " \n\t ****branch_length_mode='input' or 'marginal'", 0, warn=True)
        self.tree.root.up = None
        self.tree.root.dist2root = 0.0
        if not own_prepare:
            self._prepare_nodes()
        elif d2r is None:
            _set_dist2root(layout, lengths)
        return ttconf.SUCCESS

    def optimal_branch_length(self, node):
        """One branch: device pair histogram and Brent (treetime/treeanc.py:1244-1270)."""
        if node.up is None:
            return self.one_mutation
        if node.cseq is None and not node.clades:
            raise MissingDataError("TreeAnc.optimal_branch_length: terminal node alignments required; sequence is "
                                   "missing for leaf: '%s'." % node.name)
        pairs, mult = engine.state_pair(self.gtr, node.up.cseq, node.cseq,
                                        self.data.multiplicity(mask=getattr(node, "mask", None)), self.ignore_gaps)
        node.branch_state = {"pair": pairs, "multiplicity": mult}
        return engine.optimal_t_compressed(self.gtr, pairs, mult)

    def _profile_branch_groups(self, nodes, sess=None):
        """The profile-pair arguments of the given branches, from the outgroup
        and subtree profiles of the last marginal reconstruction: one group for
        internal nodes (child rows in the partials) and one for tips (child
        profiles from their codes), as (positions in `nodes`, node ids,
        outgroup buffer, parent rows, child rows, partials buffer); the ids and
        rows are numpy arrays (int32, int64, int64)."""
        last = getattr(self, "_last", None)
        if last is not None and last[0] == "marginal" and last[1].get("_outgroups") is not None:
            last[1]["_outgroups"]()  # rows formed on request (engine.outgroups)
        if last is None or last[0] != "marginal" or last[1].get("outgroup") is None:
            raise Exception("marginal ancestral inference needs to be performed first!")
        out = last[1]
        layout = (sess or self._get_session())["layout"]
        P = self.data.compressed_length
        ks = np.fromiter(map(layout.local.__getitem__, map(id, nodes)), dtype=np.int64, count=len(nodes))
        tip = ks >= layout.n_int
        for sel, pp, tips in ((~tip, out["outgroup"], False), (tip, out["tip_outgroup"], True)):
            idx = np.flatnonzero(sel)
            if idx.size == 0:
                continue
            kk = ks[idx]
            pp_row = ((kk - layout.n_int) if tips else kk) * P
            pc_row = np.full(idx.size, -1, np.int64) if tips else kk * P
            yield idx, kk.astype(np.int32), pp, pp_row, pc_row, out["partial"]

    def _device_branch_groups(self, nodes, sess):
        """_profile_branch_groups with the node ids and row offsets on the device, all uploaded
        before the caller launches anything; kept by the session while the same branches are
        asked for again (the TreeTime loops ask for every branch at every iteration)."""
        groups = list(self._profile_branch_groups(nodes, sess))
        cache = sess.get("branch_groups")
        if cache is not None and len(cache) == len(groups) and all(
                np.array_equal(c[0], g[1]) for c, g in zip(cache, groups)):
            dev_idx = [c[1] for c in cache]
        else:
            dev = sess["forest"].device
            dev_idx = [(engine._to_dev(kk, dev), engine._to_dev(pp_row, dev), engine._to_dev(pc_row, dev))
                       for idx, kk, pp, pp_row, pc_row, pc in groups]
            sess["branch_groups"] = [(g[1], d) for g, d in zip(groups, dev_idx)]
        return [(idx, d[0], pp, d[1], pc, d[2]) for (idx, kk, pp, pp_row, pc_row, pc), d in zip(groups, dev_idx)]

    def _marginal_branch_lengths(self, nodes, tol):
        """Profile-mode Brent for the given nodes in one device pass, from the
        outgroup and subtree profiles of the last marginal reconstruction."""
        sess = self._get_session()
        model = engine.model_for(self.gtr, getattr(self, "device", None))
        res = np.zeros(len(nodes))
        info = np.zeros(len(nodes), dtype=np.int32)
        # both branch groups are queued before either result is read back; their index arrays
        # go up first (a synchronous upload after a launch would wait for that launch)
        pending = []
        for idx, d_kk, pp, d_pp_row, pc, d_pc_row in self._device_branch_groups(nodes, sess):
            t, inf = engine.optimal_t_profiles_dev(sess["forest"], model, d_kk, pp, d_pp_row, pc, d_pc_row,
                                                   self._gpu_precision(), self.gtr.gap_index, True, tol)
            pending.append((idx, t, inf))
        for idx, t, inf in pending:
            res[idx] = t.cpu().numpy()
            info[idx] = inf.cpu().numpy()
        if (info == -1).any():
            engine.check(engine._lib.TT_ERR_BRACKET, "optimal_marginal_branch_length")
        return res

    def branch_length_grids(self, nodes=None, branch_length_mode="marginal", n_grid_points=None,
                            one_mutation=None):
        """For each branch, the grid of branch lengths and -log P(data | t) on
        it: the two arrays TreeTime's BranchLenInterpolator tabulates per node
        in ClockTree.init_date_constraints (treetime/branch_len_interpolator.py:
        36-125, treetime/clock_tree.py:343-368), for all branches in one device
        launch.  'marginal' evaluates the profile pairs of the last marginal
        reconstruction (GTR.prob_t_profiles with the node's mask), 'joint' the
        state-pair counts of the last reconstruction (GTR.prob_t_compressed).
        Returns {node: (grid, neg_log_p)}; grid points follow the node's
        mutation_length and `one_mutation` (default self.one_mutation)."""
        if branch_length_mode not in ("marginal", "joint"):
            raise Exception("unknown branch length mode! " + str(branch_length_mode))
        n_grid_points = ttconf.BRANCH_GRID_SIZE if n_grid_points is None else n_grid_points
        one_mutation = self.one_mutation if one_mutation is None else one_mutation
        if nodes is None:
            nodes = [n for n in self.tree.find_clades() if n.up is not None]
        for n in nodes:
            if n.up is None:
                raise Exception("Cannot create branch length interpolator for the root node.")
        if not nodes:
            return {}
        padded, lengths = engine.branch_len_grids([n.mutation_length for n in nodes], one_mutation, n_grid_points)
        sess = self._get_session()
        dev = sess["forest"].device
        logp = np.empty(padded.shape)
        if branch_length_mode == "marginal":
            model = engine.model_for(self.gtr, getattr(self, "device", None))
            groups = self._device_branch_groups(nodes, sess)  # uploads before any launch
            grids = [engine._to_dev(padded[g[0]], dev) for g in groups]
            pending = [(idx, engine.prob_t_profiles_grid_dev(sess["forest"], model, d_kk, pp, d_pp_row, pc, d_pc_row,
                                                             self._gpu_precision(), self.gtr.gap_index, True, grid))
                       for (idx, d_kk, pp, d_pp_row, pc, d_pc_row), grid in zip(groups, grids)]
            for idx, v in pending:
                logp[idx] = v.cpu().numpy()
        else:
            if not self.sequence_reconstruction:
                raise Exception("branch state pairs need to be assigned to nodes")
            sess, hist = self._pair_histograms()
            layout = sess["layout"]
            ks = engine._to_dev(np.asarray([layout.local[id(n)] for n in nodes], np.int64), dev)
            counts = engine.torch().trunc(hist)[ks].contiguous()  # TreeTime casts pair counts to int
            logp = engine.prob_t_pairs_grid(self.gtr.n_states, counts, sess["model"],
                                            engine._to_dev(padded, dev)).cpu().numpy()
        return {n: (padded[i, :lengths[i]], -logp[i, :lengths[i]]) for i, n in enumerate(nodes)}

    def optimal_marginal_branch_length(self, node, tol=1e-10):
        if node.up is None:
            return self.one_mutation
        return float(self._marginal_branch_lengths([node], tol)[0])

    # ------------------------------------------------------------ GTR inference
    def _tip_mismatch(self):
        """[tip rows, P] int32: alignment positions of each pattern where a
        tip's character differs from its compressed character (compression
        rewrites the ambiguous character in columns of one state; TreeTime
        counts a tip's mutations on its raw characters), or None."""
        d = self.data
        if getattr(d, "is_sparse", False):
            raise NotImplementedError("joint-mode GTR inference from a sparse alignment is not supported")
        name_to_row, ccodes = self._aln_index()
        f2c = np.asarray(d.full_to_compressed_sequence_map)
        if hasattr(d, "codes") and getattr(d, "sequence_names", None) is not None:
            raw = np.asarray(d.codes)
            rows = [name_to_row[k] for k in d.sequence_names]
        else:
            names = list(name_to_row)
            raw = np.stack([chars_to_codes(np.asarray(d.aln[k])) for k in names])
            rows = [name_to_row[k] for k in names]
        P = ccodes.shape[1]
        out = np.zeros((ccodes.shape[0], P), dtype=np.int64)
        for i, r in enumerate(rows):
            mm = raw[i] != ccodes[r][f2c]
            if mm.any():
                out[r] = np.bincount(f2c[mm], minlength=P)
        return out.astype(np.int32) if out.any() else None

    def _counting_branches(self):
        """Branches in TreeTime's counting order: children of the internal
        nodes in get_nonterminals() order (treetime/treeanc.py:1545-1546)."""
        return [c for n in self.tree.get_nonterminals() for c in n.clades]

    def get_branch_mutation_matrix(self, node, full_sequence=False):
        """[L, q, q] joint distribution of the states at both ends of the branch
        above `node` from the last marginal reconstruction (i child, j parent),
        computed on the device (treetime/treeanc.py:1085-1120)."""
        sess = self._get_session()
        if self.gtr.is_site_specific:
            for idx, kk, pp, pp_row, pc_row, pc in self._profile_branch_groups([node], sess):
                m = engine.branch_mutation_matrix_ss(sess["forest"], self.gtr, sess["bufs"], int(kk[0]), pp,
                                                     int(pp_row[0]), pc, int(pc_row[0]),
                                                     self._gpu_precision()).cpu().numpy()
        else:
            model = engine.model_for(self.gtr, getattr(self, "device", None))
            engine.branch_pmats(sess["forest"], model, sess["bufs"])
            p64 = sess["bufs"].cache[("p64", engine.torch().float64)]
            for idx, kk, pp, pp_row, pc_row, pc in self._profile_branch_groups([node], sess):
                m = engine.branch_mutation_matrix(sess["forest"], model, p64, 0, int(kk[0]), pp, int(pp_row[0]),
                                                  pc, int(pc_row[0]), self._gpu_precision()).cpu().numpy()
        if full_sequence:
            return m[self.data.full_to_compressed_sequence_map]
        return m

    def _substitution_counts(self, marginal):
        """(n_ija [q, q, P], T_ia [q, P]) over all branches, on the device."""
        sess = self._get_session()
        layout, forest = sess["layout"], sess["forest"]
        nodes = self._counting_branches()
        t = engine.torch()
        if marginal and self.gtr.is_site_specific:
            n_ija = T_ia = None
            for idx, d_kk, pp, d_pp_row, pc, d_pc_row in self._device_branch_groups(nodes, sess):
                n1, T1 = engine.mutation_counts_ss(forest, self.gtr, sess["bufs"], d_kk, pp, d_pp_row, pc, d_pc_row,
                                                   self._gpu_precision())
                n_ija = n1 if n_ija is None else n_ija + n1
                T_ia = T1 if T_ia is None else T_ia + T1
            return n_ija, T_ia
        if marginal:
            model = engine.model_for(self.gtr, getattr(self, "device", None))
            engine.branch_pmats(forest, model, sess["bufs"])
            p64 = sess["bufs"].cache[("p64", t.float64)]
            n_ija = T_ia = None
            for idx, d_kk, pp, d_pp_row, pc, d_pc_row in self._device_branch_groups(nodes, sess):
                n1, T1 = engine.mutation_counts(forest, model, p64, 0, d_kk, pp, d_pp_row, pc, d_pc_row,
                                                self._gpu_precision())
                n_ija = n1 if n_ija is None else n_ija + n1
                T_ia = T1 if T_ia is None else T_ia + T1
            return n_ija, T_ia
        states = sess["bufs"].cache.get(("states", t.uint8))
        if states is None:
            raise ValueError("Ancestral sequences are not yet inferred")
        ks = np.asarray([layout.local[id(n)] for n in nodes], np.int32)
        tips_states = bool(self.reconstructed_tip_sequences)
        return engine.mutation_counts_joint(forest, 0, engine._to_dev(ks, forest.device), states,
                                            engine.char_state_table(self.gtr, strict=True), tips_states,
                                            None if tips_states else self._tip_mismatch())

    def infer_gtr(self, marginal=False, site_specific=False, normalized_rate=True, fixed_pi=None, pc=5.0,
                  **kwargs):
        """GTR inference (treetime/treeanc.py:1500-1632): the substitution
        counts n_ija and times T_ia of all branches in one device launch, then
        TreeTime's fixed-point fit of the model on the host (GTR.infer or
        GTR_site_specific.infer)."""
        from .gtr import GTR, GTR_site_specific
        if site_specific and self.data.compress:
            raise TypeError("TreeAnc.infer_gtr(): sequence compression and site specific GTR models are "
                            "incompatible!")
        if not self.ok:
            raise MissingDataError("TreeAnc.infer_gtr: ERROR, sequences or tree are missing", 0)
        if marginal and self.sequence_reconstruction != "marginal":
            self._ml_anc_marginal(**kwargs)
        elif not self.sequence_reconstruction:
            self._ml_anc_joint(**kwargs)
        self.logger("TreeAnc.infer_gtr: counting mutations...", 2)
        n_ija, T_ia = self._substitution_counts(marginal)
        self.logger("TreeAnc.infer_gtr: counting mutations...done", 3)
        root = self.tree.root
        if site_specific:
            n_ija, T_ia = n_ija.cpu().numpy(), T_ia.cpu().numpy()
            if marginal:
                root_state = root.marginal_profile.T
            else:
                root_state = np.array([self.gtr.profile_map[c] for c in root.cseq]).T
            self._gtr = GTR_site_specific.infer(n_ija, T_ia, pc=pc, root_state=root_state, logger=self.logger,
                                                alphabet=self.gtr.alphabet, prof_map=self.gtr.profile_map)
        else:
            mult = self.data.multiplicity(mask=getattr(root, "mask", None))
            root_state = np.array([np.sum((root.cseq == nuc) * mult) for nuc in self.gtr.alphabet])
            self._gtr = GTR.infer(n_ija.sum(dim=-1).cpu().numpy(), T_ia.sum(dim=-1).cpu().numpy(), root_state,
                                  fixed_pi=fixed_pi, pc=pc, alphabet=self.gtr.alphabet, logger=self.logger,
                                  prof_map=self.gtr.profile_map)
        if normalized_rate:
            self.logger("TreeAnc.infer_gtr: setting overall rate to 1.0...", 2)
            if site_specific:
                self._gtr.mu /= self._gtr.average_rate().mean()
            else:
                self._gtr.mu = 1.0
        return self._gtr

    def infer_gtr_iterative(self, max_iter=10, site_specific=False, LHtol=0.1, pc=1.0, normalized_rate=False):
        """Alternate GTR inference and marginal reconstruction until the
        likelihood gain falls below LHtol (treetime/treeanc.py:1633-1676)."""
        self.infer_ancestral_sequences(marginal=True)
        old_p = np.copy(self.gtr.Pi)
        old_LH = self.sequence_LH()
        for i in range(max_iter):
            self.infer_gtr(site_specific=site_specific, marginal=True, normalized_rate=normalized_rate, pc=pc)
            self.infer_ancestral_sequences(marginal=True)
            dp = np.abs(self.gtr.Pi - old_p).mean() if self.gtr.Pi.shape == old_p.shape else np.nan
            deltaLH = self.sequence_LH() - old_LH
            old_p = np.copy(self.gtr.Pi)
            old_LH = self.sequence_LH()
            self.logger("TreeAnc.infer_gtr_iterative: iteration %d, LH=%1.2f (%1.2f), deltaP=%1.4f"
                        % (i, old_LH, deltaLH, dp), 2)
            if deltaLH < LHtol:
                self.logger("TreeAnc.infer_gtr_iterative: deltaLH=%f, stopping iteration." % deltaLH, 1)
                break
        return ttconf.SUCCESS

    def optimize_tree_marginal(self, max_iter=10, infer_gtr=False, pc=1.0, damping=0.75, LHtol=0.1,
                               site_specific_gtr=False, **kwargs):
        """treetime/treeanc.py:1297-1360, with the branches of an iteration
        optimised in one device pass."""
        self.infer_ancestral_sequences(marginal=True, **kwargs)
        oldLH = self.sequence_LH()
        for i in range(max_iter):
            if infer_gtr:
                self.infer_gtr(site_specific=site_specific_gtr, marginal=True, normalized_rate=True, pc=pc)
                self.infer_ancestral_sequences(marginal=True, **kwargs)
            old_bl = self.tree.total_branch_length()
            tol = 1e-8 + 0.01 ** (i + 1)
            root = self.tree.root
            special = len(root.clades) == 2
            nodes = [n for n in self.tree.find_clades() if n.up is not None and not (special and n.up is root)]
            new = dict(zip([id(n) for n in nodes], self._marginal_branch_lengths(nodes, tol))) if nodes else {}
            if special:
                n1, n2 = root.clades
                m1, m2 = getattr(n1, "mask", None), getattr(n2, "mask", None)
                if self._gpu_precision() == "f32" and (m1 is None or m2 is None) and not self.gtr.is_site_specific:
                    # from the FP32 rows on the device, as the serving loop does
                    new_bl = float(self._root_pair(n1, n2).optimal_t(
                        engine.model_for(self.gtr, getattr(self, "device", None)), self._last[1]["partial"],
                        self.gtr.gap_index, tol)[0].item())
                else:
                    prof_c = n1.marginal_subtree_LH
                    tmp = n2.marginal_subtree_LH * root.marginal_outgroup_LH
                    prof_p = np.einsum("ai,a->ai", tmp, 1.0 / tmp.sum(axis=1))
                    mult = self.data.multiplicity() if m1 is None or m2 is None else \
                        self.data.multiplicity(mask=m1 * m2)
                    new_bl = engine.optimal_t_compressed(self.gtr, (prof_p, prof_c), mult, profiles=True, tol=tol)
                # TreeTime's loop meets the pair at both children (treetime/treeanc.py:1318-1341) and
                # applies the damped update at each visit, the second from the first's lengths
                for _visit in range(2):
                    total_bl = n1.branch_length + n2.branch_length
                    bl_ratio = n1.branch_length / total_bl
                    update = new_bl * (1 - damping ** (i + 1)) + total_bl * damping ** (i + 1)
                    n1.branch_length = update * bl_ratio
                    n2.branch_length = update * (1 - bl_ratio)
                    n1.mutation_length = n1.branch_length
                    n2.mutation_length = n2.branch_length
            for n in nodes:
                update = new[id(n)] * (1 - damping ** (i + 1)) + n.branch_length * damping ** (i + 1)
                n.branch_length = update
                n.mutation_length = update
            self.infer_ancestral_sequences(marginal=True, **kwargs)
            LH = self.sequence_LH()
            deltaLH = LH - oldLH
            oldLH = LH
            self.logger("TreeAnc.optimize_tree_marginal: iteration %d, LH=%1.2f (%1.2f), delta branch_length=%1.4f"
                        % (i, LH, deltaLH, self.tree.total_branch_length() - old_bl), 2)
            if deltaLH < LHtol:
                break
        return ttconf.SUCCESS

    def _root_pair(self, n1, n2):
        """engine.RootPair of the session's tree (cached with the session)."""
        sess = self._get_session()
        rp = sess.get("root_pair")
        lay = sess["layout"]
        k1, k2 = lay.local[id(n1)], lay.local[id(n2)]
        if rp is None or (rp.n1, rp.n2) != (k1, k2):
            ti = sess["forest"].inputs[0]
            rp = engine.RootPair(sess["forest"], lay, k1, k2, ti.tip_codes, ti.tip_row)
            sess["root_pair"] = rp
        return rp

    def _prob_zero_reparented(self, sess, node, states):
        """Probability at distance zero of `node`'s states given its current
        parent's (a parent that replaced a collapsed one): the pair counts of
        the two reconstructed sequences (gaps ignored, node mask applied,
        truncated to integers as GTR.state_pair does), evaluated on the device.
        `states` caches the host copy of the states between calls."""
        layout = sess["layout"]
        t = engine.torch()
        if not states:
            P = self.data.compressed_length
            st = sess["bufs"].cache[("states", t.uint8)][: layout.n_nodes * P].cpu().numpy()
            states.append(st.reshape(layout.n_nodes, P))
        st = states[0]
        a = st[layout.local[id(node.up)]]
        b = st[layout.local[id(node)]]
        mask = getattr(node, "mask", None)
        mult = self.data.multiplicity() if mask is None else self.data.multiplicity(mask=mask)
        c = pair_counts(a, b, mult, self.gtr.n_states, self.gtr.gap_index, True)
        d = t.as_tensor(np.trunc(c)[None], dtype=t.float64, device=sess["forest"].device)
        return float(np.exp(engine.prob_t_pairs_batch(self.gtr.n_states, d, sess["model"], 0.0))[0])

    def prune_short_branches(self):
        """Collapse internal branches shorter than 0.1 / L whose sequences have
        probability > 0.1 at distance zero (treetime/treeanc.py:1475-1497);
        the histograms and zero-length likelihoods of all branches come from
        one device pass.  As in TreeTime, the pairs are counted with gaps
        ignored (GTR.prob_t's default), and a node whose parent was collapsed
        earlier in the same pass is compared with its new parent."""
        self.logger("TreeAnc.prune_short_branches: pruning short branches (max prob at zero)...", 1)
        sess, hist = self._pair_histograms(ignore_gaps=True)
        layout = sess["layout"]
        counts = engine.torch().trunc(hist)
        prob0 = np.exp(engine.prob_t_pairs_batch(self.gtr.n_states, counts, sess["model"], 0.0))
        states = []  # host copy of the reconstructed states, fetched when a parent changed
        changed = False
        for node in self.tree.find_clades():
            if node.up is None or not node.clades:
                continue
            k = layout.local.get(id(node))
            if k is None:
                continue
            if not node.branch_length < 0.1 * self.one_mutation:
                continue
            pk = layout.parent[k]
            if pk >= 0 and layout.nodes[pk] is node.up:
                p0 = prob0[k]
            else:
                p0 = self._prob_zero_reparented(sess, node, states)
            if p0 > 0.1:
                node.up.clades = [c for c in node.up.clades if c is not node] + node.clades
                for c in node.clades:
                    c.up = node.up
                changed = True
        if changed:
            self._session = None
