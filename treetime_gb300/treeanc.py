"""``TreeAnc`` with TreeTime's public interface, running the reconstruction
and branch-length hot path on the GPU.

Drop-in surface (treetime/treeanc.py): the constructor arguments,
``infer_ancestral_sequences`` / ``reconstruct_anc`` (marginal and joint),
``optimize_branch_lengths_joint``, ``optimal_branch_length``,
``optimal_marginal_branch_length``, ``optimize_tree`` (joint, marginal and
input branch-length modes), ``optimize_tree_marginal``,
``prune_short_branches``, ``sequence_LH``, ``ancestral_likelihood``,
``marginal_branch_profile``, ``get_reconstructed_alignment``, ``sequence``,
and the node and tree attributes TreeTime sets (``_cseq``,
``marginal_profile``, ``marginal_subtree_LH``, ``marginal_outgroup_LH``,
``branch_state``, ``branch_length``, ``mutation_length``,
``tree.sequence_LH``, ``tree.total_sequence_LH``,
``tree.sequence_marginal_LH``, ``tree.sequence_joint_LH``).

Per-node arrays are materialised from the device results on first access, so
a reconstruction of a large tree costs one kernel launch plus one copy of the
states and likelihoods.  ``precision='f32'`` selects the FP32 power-of-two
scaled kernels (FP64 per-pattern log-likelihoods); the default 'f64' follows
TreeTime's FP64 log-domain arithmetic.

Out of scope (raise NotImplementedError): Fitch parsimony, GTR inference,
sparse (VCF) alignments.
"""

import gc
import os
import sys
import time

import numpy as np

from . import config as ttconf
from . import engine
from .alphabets import MISSING_CODE, chars_to_codes, codes_to_chars, extend_profile
from .errors import MissingDataError, UnknownMethodError
from .gtr import GTR, GTR_site_specific
from .seqdata import SequenceData
from .tree import LAZY_ATTRS, Clade, Tree, iter_clades, read_newick


class Record:
    """Minimal alignment record (id, name, seq) for reconstructed alignments."""

    def __init__(self, id, seq, description=""):
        self.id = id
        self.name = id
        self.seq = seq
        self.description = description

    def __len__(self):
        return len(self.seq)


class Alignment(list):
    def get_alignment_length(self):
        return max((len(r.seq) for r in self), default=0)


class ResultStore:
    """Host view of one reconstruction's device results; node attributes are
    built from it on first access."""

    def __init__(self, tt, layout, kind, out, precision, reconstruct_tips, keep_outgroup, tip_outgroup):
        self.tt = tt
        self.layout = layout
        self.kind = kind
        self.out = out
        self.precision = precision
        self.reconstruct_tips = reconstruct_tips
        self.P = tt.data.compressed_length
        self.q = tt.gtr.n_states
        self.states = out["states"].view(-1)[: layout.n_nodes * self.P].cpu().numpy().reshape(layout.n_nodes, self.P)
        self._host = {}
        self.has_outgroup = keep_outgroup
        self.tip_outgroup = tip_outgroup

    def _fetch_buf(self, key):
        if key not in self._host:
            buf = self.out.get(key)
            self._host[key] = None if buf is None else buf.cpu().numpy()
        return self._host[key]

    def fetch(self, name, node):
        k = self.layout.local.get(id(node))
        if k is None:
            return None
        L, P, q = self.layout, self.P, self.q
        is_tip = k >= L.n_int
        if name == "_cseq":
            if is_tip and not self.reconstruct_tips:
                return None
            return self.tt.gtr.alphabet[self.states[k]]
        if self.kind != "marginal":
            return None
        if name == "marginal_profile":
            if is_tip:
                buf = self._fetch_buf("tip_posterior")
                return None if buf is None else buf[(k - L.n_int) * P:(k - L.n_int + 1) * P, :q].astype(np.float64)
            return self._fetch_buf("posterior")[k * P:(k + 1) * P, :q].astype(np.float64)
        if name == "marginal_subtree_LH":
            if is_tip:
                return self.tt._tip_profile(node)
            x = self._fetch_buf("partial")[k * P:(k + 1) * P, :q].astype(np.float64)
            if self.precision == "f32":
                x = x / x.sum(axis=1, keepdims=True)
            return x
        if name == "marginal_outgroup_LH":
            if k == L.n_int - 1:
                return self.tt._root_outgroup()
            if is_tip:
                buf = self._fetch_buf("tip_outgroup")
                return None if buf is None else buf[(k - L.n_int) * P:(k - L.n_int + 1) * P, :q].astype(np.float64)
            buf = self._fetch_buf("outgroup")
            return None if buf is None else buf[k * P:(k + 1) * P, :q].astype(np.float64)
        return None


class BranchStateStore:
    """branch_state dictionaries from the device pair histograms."""

    def __init__(self, layout, hist, alphabet_size):
        self.layout = layout
        self.hist = hist
        self.q = alphabet_size

    def fetch(self, name, node):
        if name != "branch_state":
            return None
        k = self.layout.local.get(id(node))
        if k is None or node.__dict__.get("up") is None:
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


class TreeAnc:
    """Ancestral sequence reconstruction and branch-length optimisation on one
    GPU with TreeTime's TreeAnc interface."""

    def __init__(self, tree=None, aln=None, gtr=None, fill_overhangs=True, ref=None, verbose=ttconf.VERBOSE,
                 ignore_gaps=True, convert_upper=True, seq_multiplicity=None, log=None, compress=True, seq_len=None,
                 ignore_missing_alns=False, keep_node_order=False, rng_seed=None, precision="f64", device=None,
                 **kwargs):
        if tree is None:
            raise TypeError("TreeAnc requires a tree!")
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        if ref is not None:
            raise NotImplementedError("sparse (VCF) alignments are not supported")
        self.t_start = time.time()
        self.verbose = verbose
        self.log = log
        self.ok = False
        self.data = None
        self.log_messages = set()
        self._internal_node_count = 0
        self.use_mutation_length = False
        self.ignore_gaps = ignore_gaps
        self.reconstructed_tip_sequences = False
        self.sequence_reconstruction = None
        self.ignore_missing_alns = ignore_missing_alns
        self.keep_node_order = keep_node_order
        self.rng = np.random.default_rng(seed=rng_seed)
        self.precision = precision
        self.device = device
        self._session = None
        self._topology_version = 0
        self._tree = None
        self.tree = tree
        self._gtr = None
        self.set_gtr(gtr or "JC69", **kwargs)
        self.data = SequenceData(aln, ref=ref, logger=self.logger, compress=compress, convert_upper=convert_upper,
                                 fill_overhangs=fill_overhangs, ambiguous=self.gtr.ambiguous, sequence_length=seq_len,
                                 seq_multiplicity=seq_multiplicity) if aln is not None else None
        if self.data is not None and self.gtr.is_site_specific and self.data.compress:
            raise TypeError("TreeAnc: sequence compression and site specific gtr models are incompatible!")
        if self.data is not None and self.data.aln and self.tree:
            self._check_alignment_tree_gtr_consistency()

    # ----------------------------------------------------------------- logging
    def logger(self, msg, level, warn=False, only_once=False):
        if only_once and msg in self.log_messages:
            return
        self.log_messages.add(msg)
        if level < self.verbose or (warn and level <= self.verbose):
            dt = time.time() - self.t_start
            print(("\n" if level < 2 else "") + format(dt, "4.2f") + "\t" + level * "-" + msg, file=sys.stdout)

    # ------------------------------------------------------------------- set-up
    @property
    def leaves_lookup(self):
        return self._leaves_lookup

    @property
    def gtr(self):
        return self._gtr

    @gtr.setter
    def gtr(self, value):
        if not isinstance(value, (GTR, GTR_site_specific)):
            raise TypeError("GTR instance expected")
        self._gtr = value
        self._session = None

    def set_gtr(self, in_gtr, **kwargs):
        if isinstance(in_gtr, str):
            self._gtr = GTR.standard(model=in_gtr, **kwargs)
            self._gtr.logger = self.logger
        elif isinstance(in_gtr, (GTR, GTR_site_specific)):
            self._gtr = in_gtr
            self._gtr.logger = self.logger
        else:
            self.logger("TreeAnc.gtr_setter: can't interpret GTR model", 1, warn=True)
            raise TypeError("Cannot set GTR model in TreeAnc class: GTR or string expected")
        if self._gtr.ambiguous is None:
            self.fill_overhangs = False
        self._session = None

    @property
    def aln(self):
        return self.data.aln if self.data else None

    @aln.setter
    def aln(self, in_aln):
        self.data = SequenceData(in_aln, logger=self.logger, ambiguous=self.gtr.ambiguous)
        self._session = None
        if self.tree:
            self._check_alignment_tree_gtr_consistency()

    @property
    def tree(self):
        return self._tree

    @tree.setter
    def tree(self, in_tree):
        self._tree = None
        if isinstance(in_tree, str):
            try:
                self._tree = read_newick(in_tree)
            except (ValueError, OSError):
                raise MissingDataError("TreeAnc: could not load tree! input was " + str(in_tree)[:200])
        elif hasattr(in_tree, "root") and hasattr(in_tree.root, "clades"):
            self._tree = in_tree
        else:
            raise MissingDataError("TreeAnc: could not load tree! input was " + str(in_tree))
        if self._tree.count_terminals() < 3:
            raise MissingDataError("TreeAnc: tree in %s as only %d tips. Please check your tree!"
                                   % (str(in_tree)[:80], self._tree.count_terminals()))
        warn = False
        for node in self._tree.find_clades():
            node.branch_length = node.branch_length if node.branch_length else 0.0
            if node.branch_length > ttconf.MAX_BRANCH_LENGTH:
                warn = True
            node.__dict__.pop("_cseq", None)
            node.original_length = node.branch_length
            node.mutation_length = node.branch_length
        if warn:
            self.logger("WARNING: TreeTime has detected branches that are longer than %d. TreeTime requires trees "
                        "where branch length is in units of average number of nucleotide or protein substitutions "
                        "per site." % ttconf.MAX_BRANCH_LENGTH, 0, warn=True)
        self.prepare_tree()
        if self.data:
            self._check_alignment_tree_gtr_consistency()

    @property
    def one_mutation(self):
        return 1.0 / self.data.full_length if self.data and self.data.full_length else np.nan

    @property
    def seq_len(self):
        return self.data.full_length

    @property
    def sequence_length(self):
        return self.data.full_length

    def _check_alignment_tree_gtr_consistency(self):
        """treetime/treeanc.py:389-444."""
        tips = self.tree.get_terminals()
        if len(tips) != len(self.data.aln):
            self.logger("**WARNING: Number of tips in tree (%d) differs from number of sequences in alignment (%d)**"
                        % (len(tips), len(self.data.aln)), 3, warn=True)
        failed = 0
        for l in tips:
            l.count = self.data.seq_multiplicity.get(l.name, 1.0)
        n_tips = len(tips)
        for l in self.tree.find_clades():
            l.__dict__.pop("branch_state", None)
            if l.name not in self.data.name_to_row and not l.clades:
                self.logger("***WARNING: TreeAnc._check_alignment_tree_gtr_consistency: NO SEQUENCE FOR LEAF: '%s'"
                            % l.name, 0, warn=True)
                failed += 1
                if not self.ignore_missing_alns and failed > n_tips / 3:
                    raise MissingDataError("TreeAnc._check_alignment_tree_gtr_consistency: At least 30\\% terminal "
                                           "nodes cannot be assigned a sequence!\nAre you sure the alignment belongs "
                                           "to the tree?")
        extend_profile(self.gtr, self.data.aln.values(), logger=self.logger)
        self.gtr._device_cache = None
        self._session = None
        self.ok = True

    def prepare_tree(self):
        """treetime/treeanc.py:446-459."""
        self.sequence_reconstruction = False
        self.tree.root.branch_length = 0.001
        self.tree.root.mask = None
        self.tree.root.mutation_length = self.tree.root.branch_length
        if not self.keep_node_order:
            self.tree.ladderize()
        self._prepare_nodes()
        self._leaves_lookup = {node.name: node for node in self.tree.get_terminals()}
        self._topology_version += 1
        self._session = None

    def _prepare_nodes(self):
        """treetime/treeanc.py:461-497: names NODE_%07d in preorder, up links,
        bad_branch flags, masks, distance to root."""
        root = self.tree.root
        root.up = None
        root.tt = self
        root.bad_branch = root.__dict__.get("bad_branch", False) if isinstance(root, Clade) else \
            getattr(root, "bad_branch", False)
        names = {n.name for n in self.tree.find_clades() if n.name}
        count = 0
        for clade in self.tree.get_nonterminals(order="preorder"):
            if clade.name is None:
                tmp = "NODE_" + format(count, "07d")
                while tmp in names:
                    count += 1
                    tmp = "NODE_" + format(count, "07d")
                clade.name = tmp
                names.add(tmp)
            count += 1
            for c in clade.clades:
                c.up = clade
                c.tt = self
        for clade in self.tree.find_clades(order="postorder"):
            if not clade.clades:
                clade.bad_branch = clade.__dict__.get("bad_branch", False)
            else:
                clade.bad_branch = all(c.bad_branch for c in clade.clades)
            if "mask" not in clade.__dict__:
                clade.mask = None
        self._calc_dist2root()
        self._internal_node_count = max(count, self._internal_node_count)

    def _calc_dist2root(self):
        self.tree.root.dist2root = 0.0
        for clade in self.tree.get_nonterminals(order="preorder"):
            for c in clade.clades:
                c.dist2root = clade.dist2root + c.mutation_length

    # ----------------------------------------------------------- device session
    def _masks_changed(self, sess):
        cur = {k: id(n.__dict__.get("mask")) for k, n in enumerate(sess["layout"].nodes)
               if n.__dict__.get("mask") is not None}
        return cur != sess["mask_ids"]

    def _get_session(self):
        """Device-resident schedule and inputs of the current tree (rebuilt on a
        topology, alignment, model or mask change; branch lengths are refreshed
        on every call)."""
        s = self._session
        if s is not None and not self._masks_changed(s):
            bl = engine.branch_lengths(s["layout"], self.data.full_length, self.use_mutation_length)
            self.gtr.check_branch_lengths(bl)
            s["forest"].set_branch_lengths([bl])
            return s
        layout = engine.TreeLayout(self.tree.root)
        P = self.data.compressed_length
        rows = []
        tip_row = np.full(layout.n_tip, -1, dtype=np.int32)
        for j, n in enumerate(layout.nodes[layout.n_int:]):
            r = self.data.name_to_row.get(n.name)
            if r is not None:
                tip_row[j] = r
        codes = self.data.compressed_codes
        masks, mask_ids = {}, {}
        for k, n in enumerate(layout.nodes):
            m = n.__dict__.get("mask")
            if m is not None:
                masks[k] = np.asarray(m, dtype=np.float64)
                mask_ids[k] = id(m)
        bl = engine.branch_lengths(layout, self.data.full_length, self.use_mutation_length)
        self.gtr.check_branch_lengths(bl)
        ti = engine.TreeInput(layout, codes, tip_row, self.data.multiplicity(), bl, masks=masks)
        forest = engine.Forest([ti], self.gtr.n_states, device=self.device)
        model = None if self.gtr.is_site_specific else self.gtr.device_model(self.device)
        s = dict(layout=layout, forest=forest, model=model, bufs=engine.Buffers(forest), mask_ids=mask_ids,
                 states_valid=False, tips_in_states=False)
        self._session = s
        return s

    def _tip_profile(self, node):
        if node.name in self.data.name_to_row:
            codes = self.data.compressed_codes[self.data.name_to_row[node.name]]
            lut = engine.profile_lut(self.gtr.profile_map, self.gtr.n_states)
            return lut[codes]
        return np.ones((self.data.compressed_length, self.gtr.n_states))

    def _root_outgroup(self):
        Pi = np.asarray(self.gtr.Pi)
        L = self.data.compressed_length
        return np.repeat([Pi], L, axis=0) if Pi.ndim == 1 else np.copy(Pi.T)

    def _seed_tip_states(self, sess):
        """Before the first reconstruction that includes tips, tip rows of the
        state buffer hold the alignment's states (255 for characters that are not
        states), so that changed-site counts compare against the alignment as
        TreeTime does."""
        layout = sess["layout"]
        P = self.data.compressed_length
        cs = engine.char_state_table(self.gtr)
        cs_strict = np.full(256, 255, np.uint8)
        for i, c in enumerate(self.gtr.alphabet):
            cs_strict[ord(str(c))] = i
        tip = np.full((layout.n_tip, P), 255, dtype=np.uint8)
        for j, n in enumerate(layout.nodes[layout.n_int:]):
            r = self.data.name_to_row.get(n.name)
            if r is not None:
                tip[j] = cs_strict[self.data.compressed_codes[r]]
        states = sess["bufs"].get("states", (sess["forest"].state_rows,), engine.torch().uint8)
        states[layout.n_int * P:].copy_(engine.torch().from_numpy(tip.reshape(-1)))

    def _clear_results(self):
        for n in self.tree.find_clades():
            d = n.__dict__
            for a in LAZY_ATTRS:
                d.pop(a, None)
            d.pop("_anc_src", None)
            d.pop("joint_Lx", None)
            d.pop("joint_Cx", None)
            d.pop("seq_idx", None)

    def _install(self, src, layout):
        for n in layout.nodes:
            if isinstance(n, Clade):
                n.__dict__["_anc_src"] = src
            else:  # foreign clade objects: materialise eagerly
                for a in LAZY_ATTRS:
                    v = src.fetch(a, n)
                    if v is not None:
                        setattr(n, a, v)

    # --------------------------------------------------------- reconstruction
    def reconstruct_anc(self, *args, **kwargs):
        return self.infer_ancestral_sequences(*args, **kwargs)

    def infer_ancestral_sequences(self, method="probabilistic", infer_gtr=False, marginal=False,
                                  reconstruct_tip_states=False, **kwargs):
        """treetime/treeanc.py:516-573."""
        if not self.ok:
            raise MissingDataError("TreeAnc.infer_ancestral_sequences: ERROR, sequences or tree are missing")
        self.logger("TreeAnc.infer_ancestral_sequences with method: %s, %s"
                    % (method, "marginal" if marginal else "joint"), 1)
        if method.lower() in ["ml", "probabilistic"]:
            fn = self._ml_anc_marginal if marginal else self._ml_anc_joint
        elif method.lower() in ["fitch", "parsimony"]:
            raise NotImplementedError("Fitch parsimony is not part of the GPU hot path")
        else:
            raise UnknownMethodError("Reconstruction method needs to be in ['ml', 'probabilistic', 'fitch', "
                                     "'parsimony'], got '{}'".format(method))
        if infer_gtr:
            raise NotImplementedError("GTR inference is not part of the GPU hot path")
        N_diff = fn(reconstruct_tip_states=reconstruct_tip_states, **kwargs)
        return N_diff

    def _root_draws(self, sample_from_profile):
        if sample_from_profile == "root" or sample_from_profile is True:
            if sample_from_profile is True:
                raise NotImplementedError("sampling states at every node is not supported; use 'root' or False")
            return self.rng.random(size=self.data.compressed_length)
        return None

    def _ml_anc_marginal(self, sample_from_profile=False, reconstruct_tip_states=False, debug=False,
                         keep_outgroup=True, **kwargs):
        """Marginal reconstruction on the GPU (treetime/treeanc.py:762-932)."""
        sess = self._get_session()
        layout = sess["layout"]
        count_diff = bool(self.sequence_reconstruction)
        if reconstruct_tip_states and count_diff and not self.reconstructed_tip_sequences:
            self._seed_tip_states(sess)
        draws = self._root_draws(sample_from_profile)
        if self.gtr.is_site_specific:
            out = engine.marginal_site_specific(sess["forest"], self.gtr, sess["bufs"], precision=self.precision,
                                                reconstruct_tips=reconstruct_tip_states, keep_outgroup=keep_outgroup,
                                                tip_outgroup=keep_outgroup, count_diff=count_diff,
                                                root_uniform=draws)
        else:
            out = engine.marginal(sess["forest"], sess["model"], sess["bufs"], precision=self.precision,
                                  reconstruct_tips=reconstruct_tip_states, keep_outgroup=keep_outgroup,
                                  tip_outgroup=keep_outgroup, count_diff=count_diff, root_uniform=draws)
        self._clear_results()
        P = self.data.compressed_length
        n_recon = layout.n_int - 1 + (layout.n_tip if reconstruct_tip_states else 0)
        N_diff = int(out["n_diff"][0].item()) if count_diff else P * n_recon
        store = ResultStore(self, layout, "marginal", out, self.precision, reconstruct_tip_states, keep_outgroup,
                            keep_outgroup)
        self._install(store, layout)
        self.tree.sequence_LH = out["site_lh"].cpu().numpy()
        self.tree.total_sequence_LH = float(out["tree_lh"][0].item())
        self.tree.sequence_marginal_LH = self.tree.total_sequence_LH
        self.reconstructed_tip_sequences = reconstruct_tip_states
        self.sequence_reconstruction = "marginal"
        self._last = ("marginal", out)
        return N_diff

    def _ml_anc_joint(self, sample_from_profile=False, reconstruct_tip_states=False, debug=False, **kwargs):
        """Joint reconstruction on the GPU (treetime/treeanc.py:934-1080)."""
        if self.gtr.is_site_specific:
            raise NotImplementedError("joint reconstruction with site-specific models is not supported")
        sess = self._get_session()
        layout = sess["layout"]
        count_diff = bool(self.sequence_reconstruction)
        if reconstruct_tip_states and count_diff and not self.reconstructed_tip_sequences:
            self._seed_tip_states(sess)
        draws = self._root_draws(sample_from_profile)
        out = engine.joint(sess["forest"], sess["model"], sess["bufs"], reconstruct_tips=reconstruct_tip_states,
                           count_diff=count_diff, root_uniform=draws)
        self._clear_results()
        P = self.data.compressed_length
        n_recon = layout.n_int - 1 + (layout.n_tip if reconstruct_tip_states else 0)
        N_diff = int(out["n_diff"][0].item()) if count_diff else P * n_recon
        store = ResultStore(self, layout, "joint", out, "f64", reconstruct_tip_states, False, False)
        self._install(store, layout)
        self.tree.sequence_LH = out["site_lh"].cpu().numpy()
        self.tree.sequence_joint_LH = float(out["tree_lh"][0].item())
        self.reconstructed_tip_sequences = reconstruct_tip_states
        self.sequence_reconstruction = "joint"
        self._last = ("joint", out)
        return N_diff

    # ------------------------------------------------------------ likelihoods
    def sequence_LH(self, pos=None, full_sequence=False):
        if not hasattr(self.tree, "total_sequence_LH"):
            self.logger("TreeAnc.sequence_LH: you need to run marginal ancestral inference first!", 1)
            self.infer_ancestral_sequences(marginal=True)
        if pos is not None:
            cp = self.data.full_to_compressed_sequence_map[pos] if full_sequence else pos
            return self.tree.sequence_LH[cp]
        return self.tree.total_sequence_LH

    def ancestral_likelihood(self):
        """Per-pattern log-likelihood of the current sequence assignment
        (treetime/treeanc.py:714-750); the branch matrices come from one batched
        device call."""
        nodes = [n for n in self.tree.find_clades(order="postorder")]
        ts = np.array([n.branch_length for n in nodes if n.up is not None])
        Ps = self.gtr.expQt(ts) if len(ts) else np.zeros((0,))
        idx = {s: i for i, s in enumerate(self.gtr.alphabet)}
        log_lh = np.zeros(self.data.compressed_length)
        k = 0
        for node in nodes:
            if node.up is None:
                prof = engine.profile_lut(self.gtr.profile_map, self.gtr.n_states)[chars_to_codes(node.cseq)]
                log_lh += np.log((prof * self.gtr.Pi).sum(axis=1))
                continue
            a = np.array([idx[c] for c in node.up.cseq])
            b = np.array([idx[c] for c in node.cseq])
            log_lh += np.log(Ps[k])[b, a]
            k += 1
        return log_lh

    def marginal_branch_profile(self, node):
        if node.up is None:
            raise Exception("Branch profiles can't be calculated for the root!")
        if not hasattr(node, "marginal_outgroup_LH"):
            raise Exception("marginal ancestral inference needs to be performed first!")
        return node.marginal_outgroup_LH, node.marginal_subtree_LH

    # --------------------------------------------------------- branch lengths
    def _pair_histograms(self):
        """Device pair histograms of every branch from the current states."""
        sess = self._get_session()
        layout = sess["layout"]
        if not self.reconstructed_tip_sequences:
            for n in layout.nodes[layout.n_int:]:
                if n.name not in self.data.name_to_row:
                    raise MissingDataError(
                        "TreeAnc.optimal_branch_length: terminal node alignments required; sequence is missing for "
                        "leaf: '%s'. Missing terminal sequences can be inferred from sister nodes by rerunning with "
                        "`reconstruct_tip_states=True` or `--reconstruct-tip-states`" % n.name)
        hist, _ = engine.state_pairs(sess["forest"], sess["bufs"], engine.char_state_table(self.gtr),
                                     self.gtr.gap_index, self.ignore_gaps, self.reconstructed_tip_sequences)
        return sess, hist

    def optimize_branch_len(self, **kwargs):
        return self.optimize_branch_lengths_joint(**kwargs)

    def optimize_branch_len_joint(self, **kwargs):
        return self.optimize_branch_lengths_joint(**kwargs)

    def optimize_branch_lengths_joint(self, **kwargs):
        """All branches at once: pair histograms and Brent on the GPU
        (treetime/treeanc.py:1176-1242)."""
        self.logger("TreeAnc.optimize_branch_length: running branch length optimization using jointML ancestral "
                    "sequences", 1)
        if self.tree is None or self.data is None or self.data.aln is None:
            raise MissingDataError("TreeAnc.optimize_branch_length: ERROR, alignment or tree are missing.")
        if not self.sequence_reconstruction:
            raise ValueError("Ancestral sequences are not yet inferred")
        store_old = kwargs.get("store_old", False)
        sess, hist = self._pair_histograms()
        layout = sess["layout"]
        counts = engine.torch().trunc(hist)
        t, info = engine.optimal_t_pairs(self.gtr.n_states, counts, sess["model"], tol=1e-10)
        t = t.cpu().numpy()
        info = info.cpu().numpy()
        root_k = layout.n_int - 1
        bad = [k for k in range(layout.n_nodes) if k != root_k and info[k] == -1]
        if bad:
            engine.check(engine._lib.TT_ERR_BRACKET, "optimize_branch_lengths_joint")
        hist_host = counts.cpu().numpy()
        max_bl = 0.0
        for k, node in enumerate(layout.nodes):
            if k == root_k:
                continue
            if store_old:
                node._old_length = node.branch_length
            new_len = max(0.0, float(t[k]))
            if new_len > 0.9 * ttconf.MAX_BRANCH_LENGTH:
                self.logger("WARNING: GTR.optimal_t_compressed -- The branch length seems to be very long!", 4,
                            warn=True)
            node.branch_length = new_len
            node.mutation_length = new_len
            max_bl = max(max_bl, new_len)
        bstore = BranchStateStore(layout, hist_host, self.gtr.n_states)
        for n in layout.nodes:
            if isinstance(n, Clade):
                n.__dict__.pop("branch_state", None)
                prev = n.__dict__.get("_anc_src")
                n.__dict__["_anc_src"] = _ChainedSource(prev, bstore) if prev is not None else bstore
            else:
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
        self._prepare_nodes()
        return ttconf.SUCCESS

    def optimal_branch_length(self, node):
        """One branch (device histogram + Brent)."""
        if node.up is None:
            return self.one_mutation
        if node.cseq is None and not node.clades:
            raise MissingDataError("TreeAnc.optimal_branch_length: terminal node alignments required; sequence is "
                                   "missing for leaf: '%s'." % node.name)
        pairs, mult = self.gtr.state_pair(node.up.cseq, node.cseq,
                                          pattern_multiplicity=self.data.multiplicity(mask=node.mask),
                                          ignore_gaps=self.ignore_gaps)
        node.branch_state = {"pair": pairs, "multiplicity": mult}
        return self.gtr.optimal_t_compressed(pairs, mult)

    def _marginal_branch_lengths(self, nodes, tol):
        """Profile-mode Brent for the given nodes on the device, from the outgroup
        and subtree profiles of the last marginal reconstruction."""
        kind, out = self._last
        if kind != "marginal" or out.get("outgroup") is None:
            raise Exception("marginal ancestral inference needs to be performed first!")
        sess = self._get_session()
        layout = sess["layout"]
        P = self.data.compressed_length
        node_of, pp_row, pc_row = [], [], []
        for n in nodes:
            k = layout.local[id(n)]
            node_of.append(k)
            if k >= layout.n_int:
                pp_row.append((k - layout.n_int) * P)
                pc_row.append(-1)
            else:
                pp_row.append(k * P)
                pc_row.append(k * P)
        # tips read their outgroup from the tip buffer: pass it as pp with tip rows
        int_idx = [i for i, k in enumerate(node_of) if k < layout.n_int]
        tip_idx = [i for i, k in enumerate(node_of) if k >= layout.n_int]
        res = np.zeros(len(nodes))
        info = np.zeros(len(nodes), dtype=np.int32)
        for idx, pp in ((int_idx, out["outgroup"]), (tip_idx, out["tip_outgroup"])):
            if not idx:
                continue
            t, inf = engine.optimal_t_profiles(sess["forest"], sess["model"], [node_of[i] for i in idx], pp,
                                               [pp_row[i] for i in idx], out["partial"], [pc_row[i] for i in idx],
                                               self.precision, self.gtr.gap_index, True, tol)
            res[idx] = t.cpu().numpy()
            info[idx] = inf.cpu().numpy()
        if (info == -1).any():
            engine.check(engine._lib.TT_ERR_BRACKET, "optimal_marginal_branch_length")
        return res

    def optimal_marginal_branch_length(self, node, tol=1e-10):
        if node.up is None:
            return self.one_mutation
        return float(self._marginal_branch_lengths([node], tol)[0])

    def optimize_tree_marginal(self, max_iter=10, infer_gtr=False, pc=1.0, damping=0.75, LHtol=0.1,
                               site_specific_gtr=False, **kwargs):
        """treetime/treeanc.py:1297-1360 with all branches of an iteration
        optimised in one device call."""
        if infer_gtr:
            raise NotImplementedError("GTR inference is not part of the GPU hot path")
        self.infer_ancestral_sequences(marginal=True, **kwargs)
        oldLH = self.sequence_LH()
        for i in range(max_iter):
            old_bl = self.tree.total_branch_length()
            tol = 1e-8 + 0.01 ** (i + 1)
            root = self.tree.root
            special = len(root.clades) == 2
            nodes = [n for n in self.tree.find_clades() if n.up is not None and not (special and n.up is root)]
            new = dict(zip([id(n) for n in nodes], self._marginal_branch_lengths(nodes, tol))) if nodes else {}
            if special:
                n1, n2 = root.clades
                total_bl = n1.branch_length + n2.branch_length
                bl_ratio = n1.branch_length / total_bl
                prof_c = n1.marginal_subtree_LH
                tmp = n2.marginal_subtree_LH * root.marginal_outgroup_LH
                prof_p = tmp * (1.0 / tmp.sum(axis=1))[:, None]
                if n1.mask is None or n2.mask is None:
                    mult = self.data.multiplicity()
                else:
                    mult = self.data.multiplicity(mask=n1.mask * n2.mask)
                new_bl = self.gtr.optimal_t_compressed((prof_p, prof_c), mult, profiles=True, tol=tol)
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

    def optimize_tree(self, prune_short=True, marginal_sequences=False, branch_length_mode="joint", max_iter=5,
                      infer_gtr=False, pc=1.0, method_anc="probabilistic", **kwargs):
        """treetime/treeanc.py:1384-1473."""
        if branch_length_mode == "marginal":
            self.optimize_tree_marginal(max_iter=max_iter, infer_gtr=infer_gtr, pc=pc, **kwargs)
            if prune_short:
                self.prune_short_branches()
            return ttconf.SUCCESS
        if branch_length_mode == "input":
            self.reconstruct_anc(method=method_anc, infer_gtr=infer_gtr, pc=pc, marginal=marginal_sequences,
                                 **kwargs)
            if prune_short:
                self.prune_short_branches()
            return ttconf.SUCCESS
        if branch_length_mode != "joint":
            raise UnknownMethodError("TreeAnc.optimize_tree: `branch_length_mode` should be in ['marginal', "
                                     "'joint', 'input']")
        self.reconstruct_anc(method=method_anc, infer_gtr=infer_gtr, pc=pc, marginal=marginal_sequences, **kwargs)
        self.optimize_branch_lengths_joint(store_old=False)
        n = 0
        while n < max_iter:
            n += 1
            if prune_short:
                self.prune_short_branches()
            N_diff = self.reconstruct_anc(method=method_anc, infer_gtr=False, marginal=marginal_sequences, **kwargs)
            self.logger("TreeAnc.optimize_tree: Iteration %d. #Nuc changed since prev reconstructions: %d"
                        % (n, N_diff), 2)
            if N_diff < 1:
                break
            self.optimize_branch_lengths_joint(store_old=False)
        self.tree.unconstrained_sequence_LH = float((self.tree.sequence_LH * self.data.multiplicity()).sum())
        self._prepare_nodes()
        return ttconf.SUCCESS

    def prune_short_branches(self):
        """Collapse internal branches shorter than 0.1 / L whose two sequences
        have probability > 0.1 at distance zero (treetime/treeanc.py:1475-1497);
        the pair histograms and zero-length likelihoods of all branches come
        from one device pass."""
        self.logger("TreeAnc.prune_short_branches: pruning short branches (max prob at zero)...", 1)
        sess, hist = self._pair_histograms()
        layout = sess["layout"]
        counts = engine.torch().trunc(hist)
        import ctypes as C
        tt = engine.torch()
        tz = tt.zeros(layout.n_nodes, dtype=tt.float64, device=counts.device)
        logp = tt.empty(layout.n_nodes, dtype=tt.float64, device=counts.device)
        engine.check(engine._lib.load().tt_prob_t_pairs(self.gtr.n_states, layout.n_nodes, engine._p(counts), None,
                                                        C.byref(sess["model"].struct), engine._p(tz), engine._p(logp),
                                                        engine._stream()), "tt_prob_t_pairs")
        prob0 = np.exp(logp.cpu().numpy())
        changed = False
        for node in self.tree.find_clades():
            if node.up is None or not node.clades:
                continue
            k = layout.local.get(id(node))
            if k is None:
                continue
            if node.branch_length < 0.1 * self.one_mutation and prob0[k] > 0.1:
                node.up.clades = [c for c in node.up.clades if c is not node] + node.clades
                for c in node.clades:
                    c.up = node.up
                changed = True
        if changed:
            self._session = None
            self._topology_version += 1

    # ------------------------------------------------------------------ output
    def get_reconstructed_alignment(self, reconstruct_tip_states=False):
        if (not self.sequence_reconstruction) or (reconstruct_tip_states != self.reconstructed_tip_sequences):
            self.infer_ancestral_sequences(reconstruct_tip_states=reconstruct_tip_states)
        return Alignment([Record(n.name, self.sequence(n, reconstructed=reconstruct_tip_states, as_string=True))
                          for n in self.tree.find_clades()])

    def sequence(self, node, reconstructed=False, as_string=True, compressed=False):
        """treetime/treeanc.py:1770-1815."""
        if isinstance(node, str):
            if node in self.leaves_lookup:
                node = self.leaves_lookup[node]
            else:
                raise ValueError("TreeAnc.sequence accepts strings are argument only when the node is terminal and "
                                 "present in the leave lookup table")
        if reconstructed and not self.reconstructed_tip_sequences:
            raise ValueError("TreeAnc.sequence can only return reconstructed terminal nodes if "
                             "TreeAnc.infer_ancestral_sequences was run with this the flag `reconstruct_tip_states`.")
        if compressed:
            if not reconstructed and node.name in self.data.name_to_row:
                tmp = self.data.compressed_alignment[node.name]
            else:
                tmp = node.cseq
        else:
            if not reconstructed and node.name in self.data.name_to_row:
                tmp = self.data.aln[node.name]
            elif node.cseq is not None:
                tmp = self.data.compressed_to_full_sequence(node.cseq, as_string=False)
            else:
                tmp = np.array([self.gtr.ambiguous or "N"] * self.sequence_length)
        return "".join(tmp) if as_string else np.copy(tmp)
