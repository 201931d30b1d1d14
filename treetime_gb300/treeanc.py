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

GTR inference (``infer_gtr``, ``infer_gtr_iterative``,
``get_branch_mutation_matrix``) counts substitutions on the GPU and fits the
model on the host as TreeTime does; Fitch parsimony (``method='fitch'``) runs
its passes up and down the tree on the GPU.

Sparse alignments ({name: {position: character}} with ``ref``, e.g. from a
VCF file through ``treetime_gb300.vcf.read_vcf``) are compressed as TreeTime
does and reconstructed like dense ones; joint-mode GTR inference from them is
not supported.
"""

import gc
import os
import sys
import time

import numpy as np

from . import config as ttconf
from . import engine
from .anc_gpu import GPUAncMixin
from .alphabets import chars_to_codes, extend_profile
from .errors import MissingDataError, UnknownMethodError
from .gtr import GTR, GTR_site_specific
from .seqdata import SequenceData
from .tree import Clade, read_newick


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


class TreeAnc(GPUAncMixin):
    """Ancestral sequence reconstruction and branch-length optimisation on one
    GPU with TreeTime's TreeAnc interface (host set-up here, device methods in
    GPUAncMixin)."""

    def __init__(self, tree=None, aln=None, gtr=None, fill_overhangs=True, ref=None, verbose=ttconf.VERBOSE,
                 ignore_gaps=True, convert_upper=True, seq_multiplicity=None, log=None, compress=True, seq_len=None,
                 ignore_missing_alns=False, keep_node_order=False, rng_seed=None, precision="f64", device=None,
                 threads=None, ctas_per_sm=None, warps_per_block=None, range_patterns=None, **kwargs):
        if tree is None:
            raise TypeError("TreeAnc requires a tree!")
        if precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
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
        self.threads = threads
        self.warps_per_block = warps_per_block
        self.range_patterns = range_patterns
        self.ctas_per_sm = ctas_per_sm
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
        extend_profile(self.gtr, [self.data.ref] if getattr(self.data, "is_sparse", False) else self.data.aln.values(),
                       logger=self.logger)
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
            fn = self._fitch_anc
        else:
            raise UnknownMethodError("Reconstruction method needs to be in ['ml', 'probabilistic', 'fitch', "
                                     "'parsimony'], got '{}'".format(method))
        if infer_gtr:
            self.infer_gtr(marginal=marginal, **kwargs)
        return fn(reconstruct_tip_states=reconstruct_tip_states, **kwargs)

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
        nodes = list(self.tree.find_clades(order="postorder"))
        ts = np.array([n.branch_length for n in nodes if n.up is not None])
        Ps = self.gtr.expQt(ts) if len(ts) else None
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

    def optimize_branch_len(self, **kwargs):
        return self.optimize_branch_lengths_joint(**kwargs)

    def optimize_branch_len_joint(self, **kwargs):
        return self.optimize_branch_lengths_joint(**kwargs)

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
