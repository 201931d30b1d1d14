"""Device engine: flattening of trees into the height-levelled CSR schedule,
HBM layout of a forest (one or many trees), and the calls into the CUDA
library.  torch provides device memory and the current stream; all compute
runs in the library's kernels.

Layout of a forest in device memory (see include/treetime_gb300.h):
  * per node (global id = tree node_base + local id): parent, tip row, branch
    length, mask offset; children as a CSR in clade order;
  * internal nodes of a tree are numbered by height (children before parents,
    the root last); the level offsets delimit each height;
  * tip characters as raw bytes, [tip][pattern] per tree;
  * profiles as [node][pattern][width] rows, width = q rounded up to 4
    (16-byte vector loads); states as [node][pattern] bytes.
"""

import collections
import ctypes as C
import operator
import time

import math

import numpy as np

from . import _lib
from . import config as ttconf
from ._lib import TTForest, TTJointOut, TTMarginalOut, TTModel, TTPmats, TTTree, check
from .alphabets import MISSING_CODE, profile_lut

TILE = 32
WIDTHS = {q: (q + 3) // 4 * 4 for q in range(1, 33)}

# Alphabet sizes the tree kernels (marginal, joint, site-specific marginal) are compiled for:
# nucleotides without / with gap, amino acids without / with gap, and 22 (aa + gap + X style).
COMPILED_ALPHABETS = (4, 5, 20, 21, 22)


def check_alphabet(q, site_specific=False):
    """Raise NotImplementedError for an alphabet size the tree kernels were not
    compiled for (the FP64 and FP32 site-specific kernels have no 5-state
    instance)."""
    sizes = (4, 20, 21, 22) if site_specific else COMPILED_ALPHABETS
    if q not in sizes:
        raise NotImplementedError(f"alphabet size {q} is not compiled into the tree kernels "
                                  f"(sizes {', '.join(map(str, sizes))})")

_torch = None


def torch():
    global _torch
    if _torch is None:
        import torch as t
        _torch = t
    return _torch


def require_device(device=None):
    """The CUDA library and a CUDA device are mandatory (no CPU path)."""
    t = torch()
    if not t.cuda.is_available():
        raise RuntimeError("treetime_gb300 needs a CUDA device: there is no CPU implementation of its kernels")
    _lib.load()
    dev = t.device(device) if device is not None else t.device("cuda", t.cuda.current_device())
    return dev


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch().cuda.current_stream().cuda_stream)


class Uploader:
    """Packs host arrays into one page-locked staging buffer and copies them
    to the device with a single non-blocking copy on the current stream;
    ``finish`` returns typed device views (each at a 256-byte aligned offset
    of one device buffer).  One asynchronous copy instead of one synchronous
    pageable copy per array: the latter stalls the host for milliseconds per
    array while other streams keep the GPU busy."""

    def __init__(self):
        self.items = []
        self.size = 0

    def add(self, name, arr):
        a = np.ascontiguousarray(arr)
        off = (self.size + 255) & ~255
        self.items.append((name, a, off))
        self.size = off + a.nbytes
        return self

    def finish(self, device):
        t = torch()
        stage = t.empty(max(1, self.size), dtype=t.uint8, pin_memory=True)
        host = stage.numpy()
        for _, a, off in self.items:
            host[off:off + a.nbytes] = a.view(np.uint8).reshape(-1)
        dbuf = stage.to(device, non_blocking=True)
        out = {}
        for name, a, off in self.items:
            tdt = t.from_numpy(a[:0]).dtype if a.size else t.uint8
            view = dbuf[off:off + a.nbytes].view(tdt)
            out[name] = view.view(a.shape) if a.size else view
        out["_buffer"] = dbuf
        return out


def _to_dev(arr, device, dtype=None):
    t = torch()
    a = np.ascontiguousarray(arr)
    x = t.from_numpy(a)
    if dtype is not None:
        x = x.to(dtype)
    return x.to(device, non_blocking=False)


# ----------------------------------------------------------------------------
# tree flattening
# ----------------------------------------------------------------------------
class TreeLayout:
    """Height-levelled CSR schedule of one rooted tree.

    ``nodes[k]`` is the clade with local id k: internal nodes first, sorted by
    height and then by preorder position (the root last), then tips in
    preorder (the order of ``get_terminals``)."""

    def __init__(self, root):
        pre = []
        stack = [root]
        while stack:
            n = stack.pop()
            pre.append(n)
            ch = n.clades
            for i in range(len(ch) - 1, -1, -1):
                stack.append(ch[i])
        pos = {id(n): i for i, n in enumerate(pre)}
        height = {}
        for n in reversed(pre):  # reverse preorder: children before parents
            height[id(n)] = 0 if not n.clades else 1 + max(height[id(c)] for c in n.clades)
        internal = [n for n in pre if n.clades]
        tips = [n for n in pre if not n.clades]
        internal.sort(key=lambda n: (height[id(n)], pos[id(n)]))
        self.nodes = internal + tips
        self.n_int = len(internal)
        self.n_tip = len(tips)
        self.root = root
        local = {id(n): k for k, n in enumerate(self.nodes)}
        self.local = local
        N = len(self.nodes)
        h = np.array([height[id(n)] for n in internal], dtype=np.int64)
        self.n_levels = int(h[-1]) if len(h) else 0
        # level_off[h-1] .. level_off[h]: internal nodes of height h
        self.level_off = np.searchsorted(h, np.arange(1, self.n_levels + 2), side="left").astype(np.int32)
        self.parent = np.full(N, -1, dtype=np.int32)
        counts = np.zeros(N + 1, dtype=np.int32)
        child_idx = []
        for k, n in enumerate(self.nodes):
            counts[k + 1] = len(n.clades)
            for c in n.clades:
                child_idx.append(local[id(c)])
                self.parent[local[id(c)]] = k
        self.child_off = np.cumsum(counts).astype(np.int32)
        self.child_idx = np.array(child_idx, dtype=np.int32)
        self.preorder_local = np.array([local[id(n)] for n in pre], dtype=np.int64)

    @property
    def n_nodes(self):
        return self.n_int + self.n_tip


def branch_lengths(layout, full_length, use_mutation_length=False):
    """Branch length used by the model: max(1e-3 / L, length)
    (TreeAnc._branch_length_to_gtr, treetime/treeanc.py:752-760).  Python's
    max keeps its first argument when the comparison with a NaN is false, so a
    NaN length becomes the floor there; np.fmax does the same."""
    attr = "mutation_length" if use_mutation_length else "branch_length"
    # None (no length) becomes NaN here and the floor below, as `or 0.0` would make it
    bl = np.array(list(map(operator.attrgetter(attr), layout.nodes)), dtype=np.float64)
    return length_floor(bl, full_length)


def length_floor(bl, full_length):
    """max(1e-3 / L, length) of an array of lengths (NaN becomes the floor)."""
    return np.fmax(ttconf.MIN_BRANCH_LENGTH * (1.0 / full_length), bl)


# ----------------------------------------------------------------------------
# models
# ----------------------------------------------------------------------------
class DeviceModel:
    """FP64 device copies of one or several standard GTR models (stacked) and
    the character -> profile table of their (shared) alphabet."""

    def __init__(self, gtrs, device=None, profile_map=None):
        if not isinstance(gtrs, (list, tuple)):
            gtrs = [gtrs]
        dev = require_device(device)
        self.device = dev
        self.gtrs = list(gtrs)
        q = gtrs[0].n_states
        for g in gtrs:
            if g.n_states != q:
                raise ValueError("all models of a forest need the same alphabet size")
        self.q = q
        self.V = _to_dev(np.stack([g.v for g in gtrs]).astype(np.float64), dev)
        self.Vinv = _to_dev(np.stack([g.v_inv for g in gtrs]).astype(np.float64), dev)
        self.lam = _to_dev(np.stack([g.eigenvals for g in gtrs]).astype(np.float64), dev)
        self.mu = _to_dev(np.array([float(g.mu) for g in gtrs], dtype=np.float64), dev)
        self.pi = _to_dev(np.stack([g.Pi for g in gtrs]).astype(np.float64), dev)
        pm = profile_map if profile_map is not None else gtrs[0].profile_map
        self.lut_host = profile_lut(pm, q)
        self.lut = _to_dev(self.lut_host, dev)
        self.lut_log2 = _to_dev(log_lut_pairs(self.lut_host, WIDTHS[q]), dev)
        self.logpi2 = _to_dev(log_pi_pairs(np.stack([g.Pi for g in gtrs]), WIDTHS[q]), dev)
        self.struct = TTModel(len(gtrs), q, _p(self.V), _p(self.Vinv), _p(self.lam), _p(self.mu), _p(self.pi),
                              _p(self.lut), _p(self.lut_log2), _p(self.logpi2))


def float_pairs(x):
    """FP64 values as FP32 pairs (hi, lo) with hi + lo equal to x to ~48 bits."""
    x = np.asarray(x, dtype=np.float64)
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def log_lut_pairs(lut, w):
    """[256][2][w] FP32 pairs of log(max(lut, 1e-12)) with non-finite values
    set to -1e10: the tips' log profiles of the joint reconstruction
    (treetime/treeanc.py:971-978)."""
    with np.errstate(divide="ignore", invalid="ignore"):
        lg = np.log(np.maximum(lut, ttconf.TINY_NUMBER))
    lg[~np.isfinite(lg)] = -ttconf.BIG_NUMBER
    hi, lo = float_pairs(lg)
    out = np.zeros((lut.shape[0], 2, w), dtype=np.float32)
    out[:, 0, :lut.shape[1]] = hi
    out[:, 1, :lut.shape[1]] = lo
    return out


def log_pi_pairs(pi, w):
    """[n_models][2][w] FP32 pairs of log(pi) (the joint reconstruction's root
    prior, treetime/treeanc.py:1021-1023); log 0 is (-inf, 0)."""
    pi = np.asarray(pi, dtype=np.float64)
    with np.errstate(divide="ignore"):
        lg = np.log(pi)
    hi, lo = float_pairs(lg)
    lo[~np.isfinite(lg)] = 0.0
    out = np.zeros((pi.shape[0], 2, w), dtype=np.float32)
    out[:, 0, :pi.shape[1]] = hi
    out[:, 1, :pi.shape[1]] = lo
    return out


# DeviceModels of recently used GTR objects, least recently used first.  An entry holds its GTR
# (DeviceModel.gtrs), so the id it is filed under cannot be reused by another object while the
# entry exists; the bound keeps a long-running server that sees a new model per request from
# holding every model it has seen.
_MODEL_CACHE = collections.OrderedDict()
MODEL_CACHE_SIZE = 256
# hits and builds of the device-model caches (DeviceModel, site-specific FP32 tables)
CACHE_STATS = collections.Counter()


def model_key(gtr):
    """Identity of a model's numbers: changes whenever its rates, frequencies or
    profile map change."""
    return (id(gtr), id(gtr.v), id(gtr.v_inv), id(gtr.eigenvals), float(np.sum(gtr.mu)), id(gtr.Pi),
            len(gtr.profile_map))


def model_for(gtr, device=None):
    """Cached DeviceModel of any object with TreeTime's GTR attributes."""
    dev = require_device(device)
    key = (model_key(gtr), str(dev))
    m = _MODEL_CACHE.get(id(gtr))
    if m is None or m[0] != key:
        m = (key, DeviceModel(gtr, dev))
        _MODEL_CACHE[id(gtr)] = m
        CACHE_STATS["model_build"] += 1
    else:
        CACHE_STATS["model_hit"] += 1
    _MODEL_CACHE.move_to_end(id(gtr))
    while len(_MODEL_CACHE) > MODEL_CACHE_SIZE:
        _MODEL_CACHE.popitem(last=False)
    return m[1]


def check_exp(gtr, t):
    """TreeTime raises ValueError when some mu*lambda*t exceeds 10
    (treetime/gtr.py:1042-1047); checked on the host before launching."""
    t = np.asarray(t, dtype=np.float64)
    if t.size == 0:
        return
    lam = np.asarray(gtr.eigenvals, dtype=np.float64)
    mu = np.asarray(gtr.mu, dtype=np.float64)
    top = float(np.max(mu * lam)) if lam.ndim == 1 else float(np.max(mu[None, :] * lam))
    if getattr(gtr, "is_site_specific", False) and getattr(gtr, "approximate", False):
        return
    if top > 0 and top * float(np.max(t)) > 10:
        raise ValueError("Error in computing exp(Q * t): Q has positive eigenvalues or the branch length t is too "
                         "large. This is most likely caused by incorrect input data.")


def site_matrices(gtr):
    """(lambda [L, q], V [L, q, q], V^-1 [L, q, q]) of a site-specific model,
    from TreeTime's layouts eigenvals [q, L], v [q, q, L], v_inv [q, q, L]."""
    lam = np.ascontiguousarray(np.asarray(gtr.eigenvals).T)
    V = np.ascontiguousarray(np.transpose(gtr.v, (2, 1, 0)))
    Vi = np.ascontiguousarray(np.transpose(gtr.v_inv, (2, 1, 0)))
    return lam, V, Vi


def site_grid(gtr):
    """Time grid of the interpolated expQt (treetime/gtr_site_specific.py:336-343)."""
    if hasattr(gtr, "t_grid"):
        return np.asarray(gtr.t_grid, dtype=np.float64)
    if hasattr(gtr, "expQt_interpolator"):
        return np.asarray(gtr.expQt_interpolator.x, dtype=np.float64)
    rs = gtr.average_rate().mean()
    return (1.0 / rs) * np.concatenate((np.linspace(0, 0.1, 11)[:-1], np.linspace(0.1, 1, 21)[:-1],
                                        np.linspace(1, 5, 21)[:-1], np.linspace(5, 10, 11)))


def prob_t_pairs_batch(q, counts, model, t):
    """log P of every branch's pair counts at one branch length t (device)."""
    tt = torch()
    n = counts.shape[0]
    d_t = tt.full((n,), float(t), dtype=tt.float64, device=counts.device)
    out = tt.empty(n, dtype=tt.float64, device=counts.device)
    check(_lib.load().tt_prob_t_pairs(q, n, _p(counts), None, C.byref(model.struct), _p(d_t), _p(out), _stream()),
          "tt_prob_t_pairs")
    return out.cpu().numpy()


def char_state_table(gtr, strict=False):
    """byte -> state index of the alphabet; TreeTime's state_pair leaves
    non-alphabet characters out for alphabets below 10 states and counts them
    as state 1 for larger ones (treetime/gtr.py:674-707).  strict: every
    non-alphabet character is 255 (GTR.state_index lookups, as in
    TreeAnc.infer_gtr)."""
    tab = np.full(256, 255, dtype=np.uint8)
    if len(gtr.alphabet) >= 10 and not strict:
        tab[:] = 1
    for i, c in enumerate(gtr.alphabet):
        tab[ord(str(c))] = i
    return tab


# ----------------------------------------------------------------------------
# forest
# ----------------------------------------------------------------------------
class TreeInput:
    """One tree's inputs: layout, tip rows (compressed codes), multiplicities,
    branch lengths, masks {local id: per-pattern array}, model index."""

    def __init__(self, layout, tip_codes, tip_row, mult, bl, masks=None, model=0):
        self.layout = layout
        self.tip_codes = np.ascontiguousarray(tip_codes, dtype=np.uint8)  # [rows, P]
        self.tip_row = np.asarray(tip_row, dtype=np.int32)                # per tip local (len n_tip)
        self.mult = np.asarray(mult, dtype=np.float64)
        self.bl = np.asarray(bl, dtype=np.float64)
        self.masks = masks or {}
        self.model = model

    @property
    def n_patterns(self):
        return len(self.mult)


class Forest:
    """Device-resident schedule and inputs of a list of trees, plus the
    C-ABI struct that points at them."""

    def __init__(self, inputs, q, device=None, warps_per_block=None, max_blocks=0, threads=None,
                 ctas_per_sm=1, range_patterns=None, ranges_per_sm=1):
        t_build = time.perf_counter()
        dev = require_device(device)
        self.device = dev
        self.inputs = list(inputs)
        self.q = q
        self.w = WIDTHS[q]
        trees = np.zeros(len(inputs), dtype=[(n, np.int64) for n in
                                             ("node_base", "level_base", "pat_base", "tip_base", "prof_base",
                                              "tipprof_base", "state_base")] +
                         [(n, np.int32) for n in ("n_int", "n_tip", "n_levels", "n_patterns", "model",
                                                   "reserved")])
        node_base = level_base = pat_base = tip_base = prof_base = tipprof_base = state_base = 0
        lev, coff, cidx, par, trow, bl, mult, codes, moff, mvals = [], [], [], [], [], [], [], [], [], []
        mask_elems = 0
        child_base = 0
        work = []
        recs, pairs, pslots = [], [], []
        for t, ti in enumerate(inputs):
            L = ti.layout
            P = ti.n_patterns
            trees[t] = (node_base, level_base, pat_base, tip_base, prof_base, tipprof_base, state_base,
                        L.n_int, L.n_tip, L.n_levels, P, ti.model, 0)
            lev.append(L.level_off)
            coff.append(L.child_off[:-1] + child_base)
            cidx.append(L.child_idx)
            rec = np.zeros((L.n_nodes, 4), dtype=np.int32)
            rec[:, 0] = L.child_off[:-1] + child_base
            rec[:, 1] = L.child_off[1:] + child_base
            rec[:, 2] = L.parent
            rec[:, 3] = -1
            rec[L.n_int:, 3] = ti.tip_row
            pair = np.full((L.n_nodes, 4), -1, dtype=np.int32)
            binary = np.flatnonzero((L.child_off[1:] - L.child_off[:-1]) == 2)
            c0 = L.child_idx[L.child_off[binary]]
            c1 = L.child_idx[L.child_off[binary] + 1]
            pair[binary, 0] = c0
            pair[binary, 1] = rec[c0, 3]
            pair[binary, 2] = c1
            pair[binary, 3] = rec[c1, 3]
            recs.append(rec)
            pairs.append(pair)
            ps = np.full(L.n_nodes, -1, dtype=np.int32)
            ps[c0] = 2 * (node_base + binary)
            ps[c1] = 2 * (node_base + binary) + 1
            pslots.append(ps)
            child_base += len(L.child_idx)
            par.append(L.parent)
            tr = np.full(L.n_nodes, -1, dtype=np.int32)
            tr[L.n_int:] = ti.tip_row
            trow.append(tr)
            bl.append(ti.bl)
            mult.append(ti.mult)
            codes.append(ti.tip_codes.reshape(-1))
            mo = np.full(L.n_nodes, -1, dtype=np.int64)
            for k, arr in ti.masks.items():
                mo[k] = mask_elems
                mvals.append(np.asarray(arr, dtype=np.float64))
                mask_elems += P
            moff.append(mo)
            for p0 in range(0, P, TILE):
                work.append((L.n_nodes * min(TILE, P - p0), t, p0))
            node_base += L.n_nodes
            level_base += len(L.level_off)
            pat_base += P
            tip_base += ti.tip_codes.size
            prof_base += L.n_int * P
            tipprof_base += L.n_tip * P
            state_base += L.n_nodes * P
        total_children = sum(len(c) for c in cidx)
        child_off = np.concatenate(coff + [np.array([total_children], dtype=np.int32)]).astype(np.int32)
        work.sort(key=lambda w: -w[0])
        self.work_host = np.array([(t, p0) for _, t, p0 in work], dtype=np.int32).reshape(-1, 2)
        sms = _lib.load().tt_device_sm_count()
        # FP32 kernel: one CTA per pattern range, one lane per pattern up to 5 states, four for
        # 20+.  Range widths make the ranges of the forest fill the GPU once (ranges_per_sm
        # CTAs per SM): each tree gets the width whose node x pattern work is one CTA's share.
        lanes_per_pattern = 4 if q >= 20 else 1
        if q != 4:
            threads = 512  # the only CTA size compiled for 5 and 20+ states
        elif threads is None:
            threads = 1024
        if threads not in (512, 1024):
            raise ValueError("threads must be 512 or 1024")
        if ctas_per_sm not in (1, 2):
            raise ValueError("ctas_per_sm must be 1 or 2")
        self.lanes_per_pattern = lanes_per_pattern
        self.threads = threads
        self.ctas_per_sm = ctas_per_sm if (q == 4 and threads == 512) else 1
        max_np = threads // lanes_per_pattern
        unit = 32 // lanes_per_pattern if lanes_per_pattern > 1 else 1
        slots = max(1, sms * max(1, int(ranges_per_sm)))
        total = sum(ti.layout.n_nodes * ti.n_patterns for ti in inputs)
        # ranges per tree: when the trees fit in the slots, shares of the slots proportional to
        # their node x pattern work (largest remainders, at least one each), so that the ranges
        # fill the GPU once without a second wave; otherwise ranges of about one slot's share
        shares = None
        if not range_patterns and 0 < len(inputs) <= slots and total > 0:
            exact = [slots * ti.layout.n_nodes * ti.n_patterns / total for ti in inputs]
            shares = [max(1, int(x)) for x in exact]
            left = slots - sum(shares)
            for t in sorted(range(len(inputs)), key=lambda t: -(exact[t] - int(exact[t]))):
                if left <= 0:
                    break
                shares[t] += 1
                left -= 1
        ranges, widths = [], []
        for t, ti in enumerate(inputs):
            P, N = ti.n_patterns, ti.layout.n_nodes
            if range_patterns:
                want = int(range_patterns)
            elif shares is not None:
                want = int(math.ceil(P / max(1, min(shares[t], P))))
            else:
                want = int(math.ceil(total / slots / max(1, N)))
            want = max(1, min(want, P, max_np))
            if unit > 1:
                want = min(max_np, -(-want // unit) * unit)
                starts = list(range(0, P, want))
                ws = [want] * len(starts)
            else:
                n_r = -(-P // want)
                if shares is not None:  # exactly the tree's share (widths differ by at most one)
                    n_r = max(n_r, min(shares[t], P))
                base_w, extra = divmod(P, n_r)
                ws = [base_w + (1 if r < extra else 0) for r in range(n_r)]
                starts = list(np.cumsum([0] + ws[:-1]))
            widths.append(max(ws))
            for p0, w_ in zip(starts, ws):
                ranges.append((N * min(w_, P - p0), t, int(p0), int(w_)))
        ranges.sort(key=lambda r: -r[0])
        self.work_f32_host = np.array([(t, p0, w_, 0) for _, t, p0, w_ in ranges], dtype=np.int32).reshape(-1, 4)
        self.trees_host = trees
        self.max_model = int(max((ti.model for ti in inputs), default=0))
        t_up = time.perf_counter()
        self.n_nodes = node_base
        self.n_patterns = pat_base
        self.prof_rows = prof_base
        self.tip_rows = tipprof_base
        self.state_rows = state_base
        up = Uploader()
        up.add("trees", trees.view(np.uint8)).add("level", np.concatenate(lev).astype(np.int32))
        up.add("child_off", child_off)
        up.add("child_idx", np.concatenate(cidx).astype(np.int32) if total_children else np.zeros(1, np.int32))
        up.add("parent", np.concatenate(par)).add("tip_row", np.concatenate(trow))
        self.bl_host = np.concatenate(bl)
        up.add("bl", self.bl_host).add("mult", np.concatenate(mult))
        # a single tree's tip codes already in page-locked memory (TreeInput.tip_codes_pinned, a torch
        # uint8 tensor) are copied on their own; otherwise they join the staging buffer
        pinned = getattr(inputs[0], "tip_codes_pinned", None) if len(inputs) == 1 else None
        if pinned is None:
            up.add("codes", codes[0] if len(codes) == 1 else (np.concatenate(codes) if codes
                                                               else np.zeros(1, np.uint8)))
        self.has_masks = mask_elems > 0
        if self.has_masks:
            up.add("mask_off", np.concatenate(moff)).add("masks", np.concatenate(mvals))
        up.add("work", self.work_host).add("work_f32", self.work_f32_host)
        up.add("node_rec", np.concatenate(recs)).add("child_pair", np.concatenate(pairs))
        up.add("pair_slot", np.concatenate(pslots))
        d = up.finish(dev)
        self._dev_buffer = d["_buffer"]
        self.d_trees, self.d_level, self.d_child_off = d["trees"], d["level"], d["child_off"]
        self.d_child_idx, self.d_parent, self.d_tip_row = d["child_idx"], d["parent"], d["tip_row"]
        if pinned is None:
            self.d_codes = d["codes"]
        else:
            self.d_codes = torch().empty(max(1, pinned.numel()), dtype=torch().uint8, device=dev)
            self.d_codes[:pinned.numel()].copy_(pinned, non_blocking=True)
        self.d_bl, self.d_mult = d["bl"], d["mult"]
        self.d_mask_off = d.get("mask_off")
        self.d_masks = d.get("masks")
        self.d_work, self.d_work_f32 = d["work"], d["work_f32"]
        self.d_node_rec, self.d_child_pair, self.d_pair_slot = d["node_rec"], d["child_pair"], d["pair_slot"]
        if warps_per_block is None:
            warps_per_block = 16 if len(self.work_host) < 2 * sms else 8
        self.struct = TTForest(
            len(inputs), q, self.w, int(max((ti.layout.n_levels for ti in inputs), default=0)),
            self.n_nodes, self.n_patterns, _p(self.d_trees), _p(self.d_level), _p(self.d_child_off),
            _p(self.d_child_idx), _p(self.d_parent), _p(self.d_tip_row), _p(self.d_mask_off), _p(self.d_masks),
            _p(self.d_bl), _p(self.d_codes), _p(self.d_mult), _p(self.d_work), len(self.work_host),
            warps_per_block, max_blocks, lanes_per_pattern, _p(self.d_work_f32), len(self.work_f32_host),
            0, _p(self.d_node_rec), _p(self.d_child_pair), _p(self.d_pair_slot), threads, self.ctas_per_sm)
        self.build_s = (t_up - t_build, time.perf_counter() - t_up)  # host preparation, device uploads

    def set_branch_lengths(self, bl_list):
        """Replace branch lengths (same topology) without rebuilding."""
        self.bl_host = np.concatenate([np.asarray(b, dtype=np.float64) for b in bl_list])
        self.d_bl.copy_(torch().from_numpy(self.bl_host))

    def tree_slices(self, t):
        """Host slices (node, pattern, profile row, state) of tree t."""
        tr = self.trees_host[t]
        return tr


# ----------------------------------------------------------------------------
# kernels
# ----------------------------------------------------------------------------
class Buffers:
    """Device outputs of the pruning passes for a forest (reused across calls;
    one buffer per name and dtype, so FP32 and FP64 passes keep their own)."""

    def __init__(self, forest):
        self.f = forest
        self.cache = {}

    def get(self, name, shape, dtype):
        t = torch()
        key = (name, dtype)
        buf = self.cache.get(key)
        if buf is None or tuple(buf.shape) != tuple(shape) or buf.dtype != dtype:
            buf = t.empty(shape, dtype=dtype, device=self.f.device)
            self.cache[key] = buf
        return buf


def branch_pmats(forest, model, bufs, need32=False, needlog=False):
    """P(t) of every branch (FP64), with the FP32 D = P - I copies of the FP32
    marginal kernel (need32) or the log pairs of the joint kernel (needlog)."""
    t = torch()
    q, w = forest.q, forest.w
    p64 = bufs.get("p64", (forest.n_nodes, q, w), t.float64)
    p32 = bufs.get("p32", (forest.n_nodes, q, w), t.float32) if need32 else None
    p32p = bufs.get("p32_pair", (forest.n_nodes, 2, q, w), t.float32) if need32 else None
    lg2 = bufs.get("logp2", (forest.n_nodes, q, 2, w), t.float32) if needlog else None
    lg2p = bufs.get("logp2_pair", (forest.n_nodes, 2, q, 2, w), t.float32) if needlog else None
    status = bufs.get("status", (1,), t.int32)
    status.zero_()
    lib = _lib.load()
    pm = TTPmats(_p(p64), _p(p32), None, _p(p32p), _p(lg2), _p(lg2p))
    check(lib.tt_branch_pmats(C.byref(forest.struct), C.byref(model.struct), pm, _p(status), _stream()),
          "tt_branch_pmats")
    return pm, status


def _check_models(forest, model):
    if forest.max_model >= model.struct.n_models:
        raise ValueError("a tree of the forest uses model %d, the DeviceModel holds %d"
                         % (forest.max_model, model.struct.n_models))


def _check_status(status):
    s = int(status.item())
    if s:
        check(s, "kernel status")


def marginal(forest, model, bufs, precision="f64", reconstruct_tips=False, keep_outgroup=False,
             tip_outgroup=False, count_diff=False, root_uniform=None, sync=True, node_uniform=None):
    """Run the marginal pass over the forest.  Returns the dict of device
    buffers (partial, posterior, outgroup, tip_posterior, tip_outgroup, states,
    site_lh, tree_lh, n_diff)."""
    t = torch()
    lib = _lib.load()
    f32 = precision == "f32"
    dt = t.float32 if f32 else t.float64
    _check_models(forest, model)
    pm, status = branch_pmats(forest, model, bufs, need32=f32)
    w = forest.w
    out = {
        "partial": bufs.get("partial", (forest.prof_rows, w), dt),
        "posterior": bufs.get("posterior", (forest.prof_rows, w), dt),
        "outgroup": bufs.get("outgroup", (forest.prof_rows, w), dt) if keep_outgroup else None,
        "tip_posterior": bufs.get("tip_posterior", (forest.tip_rows, w), dt) if reconstruct_tips else None,
        "tip_outgroup": bufs.get("tip_outgroup", (forest.tip_rows, w), dt) if tip_outgroup else None,
        "states": bufs.get("states", (forest.state_rows,), t.uint8),
        "site_lh": bufs.get("site_lh", (forest.n_patterns,), t.float64),
        "tree_lh": bufs.get("tree_lh", (len(forest.inputs),), t.float64),
        "n_diff": bufs.get("n_diff", (len(forest.inputs),), t.int64),
    }
    out["n_diff"].zero_()
    ru = _to_dev(root_uniform, forest.device, t.float64) if root_uniform is not None else None
    nu = _to_dev(node_uniform, forest.device, t.float64) if node_uniform is not None else None
    o = TTMarginalOut(_p(out["partial"]), _p(out["posterior"]), _p(out["outgroup"]), _p(out["tip_posterior"]),
                      _p(out["tip_outgroup"]), _p(out["states"]), _p(out["site_lh"]), _p(out["tree_lh"]),
                      _p(out["n_diff"]), _p(ru), int(bool(reconstruct_tips)), int(bool(count_diff)), _p(nu))
    check(lib.tt_marginal(C.byref(forest.struct), C.byref(model.struct), C.byref(pm),
                          _lib.TT_PREC_F32 if f32 else _lib.TT_PREC_F64, C.byref(o), _p(status), _stream()),
          "tt_marginal")
    if sync:
        _check_status(status)
    out["_keep"] = (ru, nu)
    return out


def marginal_lean(forest, model, bufs, snap, reconstruct_tips=False, count_diff=False, root_uniform=None,
                  node_uniform=None, sync=True):
    """The FP32 marginal pass (alphabets up to 5 states) without the outputs nothing in the pass
    depends on: the outgroup rows (formed on request by `outgroups`) and the changed-site count
    (tt_count_changes against the states taken before the pass).  `snap` is a dict of device
    buffers owned by the caller; it receives the branch lengths the pass used ("bl") and, with
    count_diff, the states before it ("old").  Same outputs as marginal() otherwise."""
    t = torch()
    bl = snap.get("bl")
    if bl is None or bl.shape != forest.d_bl.shape:
        bl = snap["bl"] = t.empty_like(forest.d_bl)
    bl.copy_(forest.d_bl)
    snap["forest"] = forest
    states = bufs.get("states", (forest.state_rows,), t.uint8)
    if count_diff:
        old = snap.get("old")
        if old is None or old.shape != states.shape:
            old = snap["old"] = t.empty_like(states)
        old.copy_(states)
    out = marginal(forest, model, bufs, precision="f32", reconstruct_tips=reconstruct_tips, count_diff=False,
                   root_uniform=root_uniform, node_uniform=node_uniform, sync=False)
    if count_diff:
        check(_lib.load().tt_count_changes(C.byref(forest.struct), _p(snap["old"]), _p(states),
                                           int(bool(reconstruct_tips)), _p(out["n_diff"]), _stream()),
              "tt_count_changes")
    if sync:
        _check_status(bufs.get("status", (1,), t.int32))
    return out


def outgroups(forest, model, bufs, out, snap, scratch):
    """The outgroup rows (internal nodes and tips) of a pass run by marginal_lean, formed once
    into `bufs`' outgroup buffers and entered into `out`: the branch matrices of the lengths the
    pass used (snap["bl"]) into `scratch` (a Buffers of its own, so the forest's matrices stay as
    they are), then tt_outgroups_f32.  Waits for the result and checks the status."""
    if out.get("outgroup") is not None:
        return out
    t = torch()
    lib = _lib.load()
    q, w = forest.q, forest.w
    fs = TTForest.from_buffer_copy(forest.struct)  # the forest with the pass's branch lengths
    fs.bl = _p(snap["bl"])
    p64 = scratch.get("p64", (forest.n_nodes, q, w), t.float64)
    p32 = scratch.get("p32", (forest.n_nodes, q, w), t.float32)
    status = scratch.get("status", (1,), t.int32)
    status.zero_()
    check(lib.tt_branch_pmats(C.byref(fs), C.byref(model.struct), TTPmats(_p(p64), _p(p32), None, None, None, None),
                              _p(status), _stream()), "tt_branch_pmats")
    og = bufs.get("outgroup", (forest.prof_rows, w), t.float32)
    tog = bufs.get("tip_outgroup", (forest.tip_rows, w), t.float32)
    check(lib.tt_outgroups_f32(C.byref(fs), C.byref(model.struct), C.byref(TTPmats(_p(p64), _p(p32), None, None,
                                                                                   None, None)),
                               _p(out["posterior"]), _p(out["partial"]), _p(og), _p(tog), _stream()),
          "tt_outgroups_f32")
    _check_status(status)
    out["outgroup"], out["tip_outgroup"] = og, tog
    return out


class CapturedCall:
    """One call of a pass function (marginal, joint: its buffer clears and launches) captured as
    a CUDA graph, replayed with a single host call.  The kernels read the forest's device inputs
    (tip codes, branch lengths, multiplicities) at replay, so values written there in place are
    seen; the outputs are the same device buffers every time.  The function must have run on
    this forest with the same options before (buffers allocated, kernel attributes set), so that
    nothing is allocated or configured inside the capture."""

    def __init__(self, fn, *args, after=None, **kw):
        t = torch()
        self.graph = t.cuda.CUDAGraph()
        with t.cuda.graph(self.graph):
            self.out = fn(*args, sync=False, **kw)
            if after is not None:  # further work on the outputs, captured with them (copies)
                after(self.out)
        self._keep = args  # the captured launches point into these objects' device buffers

    def replay(self):
        self.graph.replay()
        return self.out


class CapturedMarginal:
    """One marginal pass over a forest captured as a CUDA graph: the buffer
    clears and the three launches (branch matrices, the pass, the per-tree
    sums) replay with a single host call and no gaps between kernels.  The
    forest's device inputs (tip codes, branch lengths, multiplicities) may be
    overwritten in place between replays; the outputs are the same device
    buffers every time (``self.out``).  Root sampling is not captured (its
    uniform draws are a per-call host input)."""

    def __init__(self, forest, model, bufs, precision="f32", reconstruct_tips=False, keep_outgroup=False,
                 tip_outgroup=False, count_diff=False):
        t = torch()
        kw = dict(precision=precision, reconstruct_tips=reconstruct_tips, keep_outgroup=keep_outgroup,
                  tip_outgroup=tip_outgroup, count_diff=count_diff)
        marginal(forest, model, bufs, sync=True, **kw)  # allocates every buffer, configures the kernels
        side = t.cuda.Stream(device=forest.device)
        side.wait_stream(t.cuda.current_stream(forest.device))
        with t.cuda.stream(side):
            marginal(forest, model, bufs, sync=False, **kw)
        t.cuda.current_stream(forest.device).wait_stream(side)
        self.graph = t.cuda.CUDAGraph()
        with t.cuda.graph(self.graph):
            self.out = marginal(forest, model, bufs, sync=False, **kw)
        self.status = bufs.get("status", (1,), t.int32)
        self._keep = (forest, model, bufs)  # the captured launches point into their device buffers

    def replay(self, sync=False):
        self.graph.replay()
        if sync:
            _check_status(self.status)
        return self.out


_SS_F32_CACHE = {}


def _ss_f32_model(forest, gtr, bufs, dev, range_width=None):
    """FP32 site-interleaved model arrays and site ranges for tt_marginal_ss_f32
    (cached per model, row width, device and range width)."""
    key = (model_key(gtr), forest.w, str(dev), range_width)
    hit = _SS_F32_CACHE.get(key)
    if hit is not None:
        CACHE_STATS["site_model_hit"] += 1
        return hit
    CACHE_STATS["site_model_build"] += 1
    t = torch()
    lam, V, Vi = site_matrices(gtr)                    # [P][q], [P][q][q], [P][q][q] (FP64)
    P, q = lam.shape
    w = forest.w
    mu = np.asarray(gtr.mu, dtype=np.float64).reshape(-1)
    mulam = mu[:, None] * lam                          # [P][q]

    def rows(x):                                       # [..., q] -> [..., w] float32, zero padded
        out = np.zeros(x.shape[:-1] + (w,), dtype=np.float32)
        out[..., :q] = x
        return out

    arrs = dict(
        V=_to_dev(np.ascontiguousarray(V.transpose(1, 2, 0).reshape(q * q, P)).astype(np.float32), dev),
        Vi=_to_dev(np.ascontiguousarray(Vi.transpose(1, 2, 0).reshape(q * q, P)).astype(np.float32), dev),
        mulam=_to_dev(rows(mulam), dev),
        pi=_to_dev(rows(np.asarray(gtr.Pi, dtype=np.float64).T), dev),
        lut=_to_dev(profile_lut(gtr.profile_map, gtr.n_states), dev))
    n_grid = 0
    if gtr.approximate:
        grid = site_grid(gtr)
        n_grid = len(grid)
        em1 = np.expm1(grid[:, None, None] * mulam[None, :, :])  # [n_grid][P][q]
        arrs["grid"] = _to_dev(grid, dev)
        arrs["em1"] = _to_dev(rows(em1), dev)
    # site ranges: about one per SM, at most 32 sites
    sms = _lib.load().tt_device_sm_count()
    width = int(min(32, max(1, range_width or math.ceil(P / max(1, sms)))))
    starts = np.arange(0, P, width)
    ranges = np.zeros((len(starts), 4), dtype=np.int32)
    ranges[:, 1] = starts
    ranges[:, 2] = np.minimum(width, P - starts)
    arrs["ranges"] = _to_dev(ranges, dev)
    arrs["struct"] = _lib.TTSSF32(P, n_grid, _p(arrs["V"]), _p(arrs["Vi"]), _p(arrs["mulam"]), _p(arrs["pi"]),
                                  _p(arrs.get("em1")), _p(arrs.get("grid")), _p(arrs["lut"]),
                                  float(gtr.rate_scale))
    if len(_SS_F32_CACHE) > 16:
        _SS_F32_CACHE.clear()
    _SS_F32_CACHE[key] = arrs
    return arrs


def marginal_site_specific(forest, gtr, bufs, precision="f64", reconstruct_tips=False, keep_outgroup=False,
                           tip_outgroup=False, count_diff=False, root_uniform=None, sync=True, range_width=None,
                           node_uniform=None):
    """Marginal pass for a GTR_site_specific model (single tree): FP64 log-domain
    kernel, or the FP32 kernel with each site range's eigenvectors in shared
    memory."""
    t = torch()
    lib = _lib.load()
    f32 = precision == "f32"
    dt = t.float32 if f32 else t.float64
    dev = forest.device
    w = forest.w
    out = {
        "partial": bufs.get("partial", (forest.prof_rows, w), dt),
        "posterior": bufs.get("posterior", (forest.prof_rows, w), dt),
        "outgroup": bufs.get("outgroup", (forest.prof_rows, w), dt) if keep_outgroup else None,
        "tip_posterior": bufs.get("tip_posterior", (forest.tip_rows, w), dt) if reconstruct_tips else None,
        "tip_outgroup": bufs.get("tip_outgroup", (forest.tip_rows, w), dt) if tip_outgroup else None,
        "states": bufs.get("states", (forest.state_rows,), t.uint8),
        "site_lh": bufs.get("site_lh", (forest.n_patterns,), t.float64),
        "tree_lh": bufs.get("tree_lh", (len(forest.inputs),), t.float64),
        "n_diff": bufs.get("n_diff", (len(forest.inputs),), t.int64),
    }
    out["n_diff"].zero_()
    status = bufs.get("status", (1,), t.int32)
    status.zero_()
    ru = _to_dev(root_uniform, dev, t.float64) if root_uniform is not None else None
    nu = _to_dev(node_uniform, dev, t.float64) if node_uniform is not None else None
    o = TTMarginalOut(_p(out["partial"]), _p(out["posterior"]), _p(out["outgroup"]), _p(out["tip_posterior"]),
                      _p(out["tip_outgroup"]), _p(out["states"]), _p(out["site_lh"]), _p(out["tree_lh"]),
                      _p(out["n_diff"]), _p(ru), int(bool(reconstruct_tips)), int(bool(count_diff)), _p(nu))
    if f32:
        arrs = _ss_f32_model(forest, gtr, bufs, dev, range_width)
        check(lib.tt_marginal_ss_f32(C.byref(forest.struct), C.byref(arrs["struct"]), _p(arrs["ranges"]),
                                     int(arrs["ranges"].shape[0]), C.byref(o), _p(status), _stream()),
              "tt_marginal_ss_f32")
    else:
        arrs = _ss_model64(gtr, bufs, dev)
        check(lib.tt_marginal_ss(C.byref(forest.struct), _p(arrs["lam"]), _p(arrs["V"]), _p(arrs["Vi"]),
                                 _p(arrs["mu"]), _p(arrs["pi"]), _p(arrs["lut"]), _p(arrs["grid"]),
                                 int(arrs["grid"].numel()), float(gtr.rate_scale), int(bool(gtr.approximate)),
                                 _lib.TT_PREC_F64, C.byref(o), _p(status), _stream()), "tt_marginal_ss")
    if sync:
        _check_status(status)
    out["_keep"] = (ru, nu)
    return out


def _ss_model64(gtr, bufs, dev, need_stack=False):
    """FP64 device arrays of a site-specific model (cached per model in the
    forest's buffers); with need_stack and TreeTime's interpolated P(t), the
    exact matrices at the grid points (tt_ss_pstack) as well."""
    key = model_key(gtr)
    cache = bufs.cache.get("ss_model")
    if cache is None or cache[0] != key:
        lam, V, Vi = site_matrices(gtr)
        arrs = dict(lam=_to_dev(lam, dev), V=_to_dev(V, dev), Vi=_to_dev(Vi, dev),
                    mu=_to_dev(np.asarray(gtr.mu, dtype=np.float64), dev),
                    pi=_to_dev(np.ascontiguousarray(gtr.Pi.T), dev),
                    lut=_to_dev(profile_lut(gtr.profile_map, gtr.n_states), dev),
                    grid=_to_dev(site_grid(gtr), dev))
        bufs.cache["ss_model"] = (key, arrs)
    arrs = bufs.cache["ss_model"][1]
    q = gtr.n_states
    L = int(arrs["mu"].numel())
    approx = bool(getattr(gtr, "approximate", False))
    if "struct" not in arrs:
        arrs["struct"] = _lib.TTSSModel(q, int(arrs["grid"].numel()), int(approx), 0, float(gtr.rate_scale),
                                        _p(arrs["lam"]), _p(arrs["V"]), _p(arrs["Vi"]), _p(arrs["mu"]),
                                        _p(arrs["pi"]), _p(arrs["lut"]), _p(arrs["grid"]), None)
    if need_stack and approx and "stack" not in arrs:
        t = torch()
        arrs["stack"] = t.empty((int(arrs["grid"].numel()), q, q, L), dtype=t.float64, device=dev)
        check(_lib.load().tt_ss_pstack(C.byref(arrs["struct"]), L, _p(arrs["stack"]), _stream()), "tt_ss_pstack")
        arrs["struct"].stack = _p(arrs["stack"])
    return arrs


def joint_site_specific(forest, gtr, bufs, reconstruct_tips=False, count_diff=False, root_uniform=None, sync=True):
    """Joint reconstruction under a GTR_site_specific model (single tree): per
    node and site log P from TreeTime's interpolated (or exact) per-site
    matrices in FP64, one launch per height level."""
    t = torch()
    lib = _lib.load()
    if len(forest.inputs) != 1:
        raise ValueError("joint reconstruction with a site-specific model takes one tree")
    dev = forest.device
    arrs = _ss_model64(gtr, bufs, dev, need_stack=True)
    lay = forest.inputs[0].layout
    w = forest.w
    out = {
        "msg": bufs.get("joint_msg", (forest.prof_rows, 2, w), t.float32),
        "cx": bufs.get("cx", (forest.prof_rows, w), t.uint8),
        "states": bufs.get("states", (forest.state_rows,), t.uint8),
        "site_lh": bufs.get("joint_site_lh", (forest.n_patterns,), t.float64),
        "tree_lh": bufs.get("joint_tree_lh", (1,), t.float64),
        "n_diff": bufs.get("n_diff", (1,), t.int64),
    }
    out["n_diff"].zero_()
    status = bufs.get("status", (1,), t.int32)
    status.zero_()
    ru = _to_dev(root_uniform, dev, t.float64) if root_uniform is not None else None
    o = TTJointOut(_p(out["msg"]), _p(out["cx"]), _p(out["states"]), _p(out["site_lh"]), _p(out["tree_lh"]),
                   _p(out["n_diff"]), _p(ru), int(bool(reconstruct_tips)), int(bool(count_diff)),
                   int(forest.prof_rows))
    lev = np.ascontiguousarray(lay.level_off, dtype=np.int32)
    check(lib.tt_joint_ss(C.byref(forest.struct), C.byref(arrs["struct"]), lev.ctypes.data_as(C.c_void_p),
                          int(lay.n_levels), int(lay.n_int), int(lay.n_tip), C.byref(o), _p(status), _stream()),
          "tt_joint_ss")
    if sync:
        _check_status(status)
    out["_keep"] = ru
    return out


def joint(forest, model, bufs, reconstruct_tips=False, count_diff=False, root_uniform=None, sync=True):
    t = torch()
    lib = _lib.load()
    _check_models(forest, model)
    pm, status = branch_pmats(forest, model, bufs, needlog=True)
    w = forest.w
    out = {
        "msg": bufs.get("joint_msg", (forest.prof_rows, 2, w), t.float32),
        "cx": bufs.get("cx", (forest.prof_rows, w), t.uint8),
        "states": bufs.get("states", (forest.state_rows,), t.uint8),
        "site_lh": bufs.get("joint_site_lh", (forest.n_patterns,), t.float64),
        "tree_lh": bufs.get("joint_tree_lh", (len(forest.inputs),), t.float64),
        "n_diff": bufs.get("n_diff", (len(forest.inputs),), t.int64),
    }
    out["n_diff"].zero_()
    ru = _to_dev(root_uniform, forest.device, t.float64) if root_uniform is not None else None
    o = TTJointOut(_p(out["msg"]), _p(out["cx"]), _p(out["states"]), _p(out["site_lh"]), _p(out["tree_lh"]),
                   _p(out["n_diff"]), _p(ru), int(bool(reconstruct_tips)), int(bool(count_diff)),
                   int(forest.prof_rows))
    check(lib.tt_joint(C.byref(forest.struct), C.byref(model.struct), C.byref(pm), C.byref(o), _p(status),
                       _stream()), "tt_joint")
    if sync:
        _check_status(status)
    out["_keep"] = ru
    return out


def state_pairs(forest, bufs, char_state, gap_state, ignore_gaps, tips_use_states):
    """[n_nodes, q, q] multiplicity-weighted (parent, child) histograms
    (char_state: the byte -> state table, host array or device tensor)."""
    t = torch()
    lib = _lib.load()
    q = forest.q
    hist = bufs.get("hist", (forest.n_nodes, q, q), t.float64)
    hist.zero_()
    cs = char_state if hasattr(char_state, "data_ptr") else _to_dev(char_state, forest.device)
    check(lib.tt_state_pairs(C.byref(forest.struct), _p(bufs.cache[("states", t.uint8)]), _p(cs), int(bool(tips_use_states)),
                             -1 if gap_state is None else int(gap_state), int(bool(ignore_gaps)), None, _p(hist),
                             _stream()), "tt_state_pairs")
    return hist, cs


def optimal_t_pairs(q, counts, model, model_of=None, tol=1e-10):
    """Brent per branch on [n, q, q] counts (device tensor) -> (t, info)."""
    t = torch()
    lib = _lib.load()
    n = counts.shape[0]
    tout = t.empty(n, dtype=t.float64, device=counts.device)
    info = t.empty(n, dtype=t.int32, device=counts.device)
    mo = None
    if model_of is not None:
        mo = model_of if hasattr(model_of, "data_ptr") else _to_dev(np.asarray(model_of, np.int32), counts.device)
    check(lib.tt_optimal_t_pairs(q, n, _p(counts), _p(mo), C.byref(model.struct), float(tol), _p(tout), _p(info),
                                 _stream()), "tt_optimal_t_pairs")
    return tout, info


def optimal_t_profiles(forest, model, node_of, pp, pp_row, pc, pc_row, precision, gap_state, ignore_gaps,
                       tol=1e-10):
    dev = forest.device
    return optimal_t_profiles_dev(forest, model, _to_dev(np.asarray(node_of, np.int32), dev), pp,
                                  _to_dev(np.asarray(pp_row, np.int64), dev), pc,
                                  _to_dev(np.asarray(pc_row, np.int64), dev), precision, gap_state, ignore_gaps, tol)


def optimal_t_profiles_dev(forest, model, d_node, pp, d_pp_row, pc, d_pc_row, precision, gap_state, ignore_gaps,
                           tol=1e-10):
    """optimal_t_profiles with the branch list (int32 node ids) and the row
    offsets (int64) already on the device: enqueues only, no host copy."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    n = int(d_node.numel())
    tout = t.empty(n, dtype=t.float64, device=dev)
    info = t.empty(n, dtype=t.int32, device=dev)
    ws, ws_bytes = _profile_workspace(forest, n, dev, precision)
    check(lib.tt_optimal_t_profiles(C.byref(forest.struct), C.byref(model.struct), n, _p(d_node), _p(pp),
                                    _p(d_pp_row), _p(pc), _p(d_pc_row),
                                    _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64,
                                    -1 if gap_state is None else int(gap_state), int(bool(ignore_gaps)), float(tol),
                                    _p(tout), _p(info), _p(ws), ws_bytes, _stream()), "tt_optimal_t_profiles")
    return tout, info


class RootPair:
    """The bifurcating root's two children as one branch (treetime/treeanc.py:
    1317-1339) on the device: Brent in profile mode between the first child's
    subtree profile and the second child's subtree profile times the root's
    outgroup (pi), normalised, from the FP32 rows of a marginal
    reconstruction.  Holds the small index arrays of one tree (uploaded once)."""

    def __init__(self, forest, layout, n1, n2, tip_codes, tip_row):
        t = torch()
        P = forest.inputs[0].n_patterns if len(forest.inputs) == 1 else None
        if P is None:
            raise ValueError("RootPair takes a forest of one tree")
        self.forest, self.n1, self.n2, self.P = forest, int(n1), int(n2), P
        dev = forest.device
        up = Uploader()
        up.add("n1", np.array([n1], np.int32))
        up.add("n1_row", np.array([n1 * P if n1 < layout.n_int else -1], np.int64))
        up.add("zero_row", np.zeros(1, np.int64))
        self.n2_is_tip = n2 >= layout.n_int
        if self.n2_is_tip:
            r = int(tip_row[n2 - layout.n_int])
            up.add("n2_codes", np.ascontiguousarray(tip_codes[r] if r >= 0 else np.zeros(P, np.uint8)))
        self.d = up.finish(dev)
        self._pp = t.empty((P, forest.w), dtype=t.float32, device=dev)

    def optimal_t(self, model, partial, gap_state, tol):
        """Device tensor [1]: the pair's optimal total length (enqueued only)."""
        t = torch()
        q, P = self.forest.q, self.P
        if not self.n2_is_tip:
            x2 = partial[self.n2 * P:(self.n2 + 1) * P, :q].to(t.float64)
        else:
            x2 = model.lut[self.d["n2_codes"].long()]
        y = x2 * model.pi[0][None, :]
        y = y / y.sum(dim=1, keepdim=True)
        self._pp.zero_()
        self._pp[:, :q].copy_(y)
        tn, _ = optimal_t_profiles_dev(self.forest, model, self.d["n1"], self._pp, self.d["zero_row"], partial,
                                       self.d["n1_row"], "f32", gap_state, True, tol)
        return tn


_PROFILE_WS = {}


def _profile_workspace(forest, n, dev, precision="f64"):
    """Device workspace of the profile-Brent and grid kernels (one slice per
    persistent CTA): FP64 kernels, the per-pattern coefficients that do not fit
    in shared memory; the FP32 Brent kernel (FP32 profiles, up to 5 states),
    the FP32 pattern rows of trees with more patterns than its shared memory
    holds.  One buffer per device and stream, grown when a call needs more."""
    t = torch()
    q = forest.q
    p_max = int(np.max(forest.trees_host["n_patterns"])) if len(forest.trees_host) else 0
    sms = _lib.load().tt_device_sm_count()
    if precision == "f32" and q <= 5 and q >= 4:
        # the kernel's shared memory: pattern rows plus one heavy-pattern mask word per 32 patterns
        cap = (100 * 1024) // ((2 * q + 1) * 4)
        while cap * (2 * q + 1) * 4 + (cap + 31) // 32 * 4 > 100 * 1024:
            cap -= 1
        if p_max <= cap or n == 0:
            return None, 0
        blocks = min(n, 2 * sms)
        per = -(-(((p_max + 3) & ~3) * (2 * q + 1) * 4) // 16) * 16
        need = blocks * per
    else:
        cap = (200 * 1024) // ((q + 1) * 8)
        over = max(0, p_max - cap)
        if over == 0 or n == 0:
            return None, 0
        blocks = min(n, sms)
        need = blocks * over * (q + 1) * 8
    key = (str(dev), t.cuda.current_stream(dev).cuda_stream)
    buf = _PROFILE_WS.get(key)
    if buf is None or buf.numel() < need // 8:
        buf = t.empty(need // 8, dtype=t.float64, device=dev)
        _PROFILE_WS[key] = buf
    return buf, int(buf.numel() * 8)


# ----------------------------------------------------------------------------
# single-call GTR API (device computations behind GTR methods)
# ----------------------------------------------------------------------------
def branch_len_grids(mutation_lengths, one_mutation, n_grid_points=ttconf.BRANCH_GRID_SIZE):
    """The branch lengths at which BranchLenInterpolator tabulates each
    branch's likelihood (treetime/branch_len_interpolator.py:36-62), for many
    branches at once: ([n, G] grids padded with -1, [n] lengths).  The numpy
    expressions are TreeTime's, applied row-wise (elementwise IEEE operations
    and a row sort), so every row is identical to TreeTime's grid: for an
    effectively zero branch (mutation_length < min(1e-5, one_mutation / 10))
    a linear ramp to 10 mutations then a quadratic one to MAX_BRANCH_LENGTH;
    otherwise points clustered at zero, a quadratic approach to the branch
    length, a quadratic tail to 4x it and a sparse tail to MAX_BRANCH_LENGTH."""
    ml = np.asarray(mutation_lengths, dtype=np.float64).reshape(-1)
    n = int(n_grid_points)
    zero = ml < np.min((1e-5, 0.1 * one_mutation))
    short = 10 * one_mutation
    zgrid = np.concatenate([short * (np.linspace(0, 1.0, n // 2)[:-1]),
                            short + (ttconf.MAX_BRANCH_LENGTH - short) * (np.linspace(0, 1.0, n // 2 + 1) ** 2)])
    m = ml[~zero][:, None]
    left = m * (1 - np.linspace(1, 0.0, n // 3) ** 2.0)
    near_zero = left[:, 1:2] * np.logspace(-20, 0, 6)[:5]
    near_zero2 = left[:, 1:2] * np.linspace(0, 1, 10)[1:-1]
    right = m + (3 * m * (np.linspace(0, 1, n // 3) ** 2))
    far = right.max(axis=1, keepdims=True) + ttconf.MAX_BRANCH_LENGTH * np.linspace(0, 1, n // 3) ** 2
    fgrid = np.concatenate((near_zero, near_zero2, left, right[:, 1:], far[:, 1:]), axis=1)
    fgrid.sort(axis=1)
    G = max(len(zgrid) if zero.any() else 0, fgrid.shape[1] if len(m) else 0)
    out = np.full((len(ml), G), -1.0)
    lengths = np.where(zero, len(zgrid), fgrid.shape[1]).astype(np.int64)
    if zero.any():
        out[zero, :len(zgrid)] = zgrid
    if len(m):
        out[~zero, :fgrid.shape[1]] = fgrid
    return out, lengths


def branch_len_grid(mutation_length, one_mutation, n_grid_points=ttconf.BRANCH_GRID_SIZE):
    """One branch's grid (see branch_len_grids)."""
    g, n = branch_len_grids([mutation_length], one_mutation, n_grid_points)
    return g[0, :n[0]]


def prob_t_profiles_grid_dev(forest, model, d_node, pp, d_pp_row, pc, d_pc_row, precision, gap_state, ignore_gaps,
                             d_grid):
    """log P(profiles | t) of each listed branch at each point of its row of
    d_grid ([n][G] device FP64): the 'marginal' BranchLenInterpolator values
    (treetime/branch_len_interpolator.py:96-105), enqueued in one launch."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    n = int(d_node.numel())
    G = int(d_grid.shape[1]) if d_grid.dim() == 2 else 0
    if d_grid.shape[0] != n:
        raise ValueError("prob_t_profiles_grid: %d grid rows for %d branches" % (d_grid.shape[0], n))
    out = t.empty((n, G), dtype=t.float64, device=dev)
    ws, ws_bytes = _profile_workspace(forest, n, dev)
    check(lib.tt_prob_t_profiles_grid(C.byref(forest.struct), C.byref(model.struct), n, _p(d_node), _p(pp),
                                      _p(d_pp_row), _p(pc), _p(d_pc_row),
                                      _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64,
                                      -1 if gap_state is None else int(gap_state), int(bool(ignore_gaps)),
                                      _p(d_grid), G, _p(out), _p(ws), ws_bytes, _stream()), "tt_prob_t_profiles_grid")
    return out


def prob_t_pairs_grid(q, counts, model, d_grid, model_of=None):
    """log P(state pairs | t) of [n, q, q] device counts at each point of the
    branch's row of d_grid: the 'joint' BranchLenInterpolator values
    (treetime/branch_len_interpolator.py:107-118)."""
    t = torch()
    lib = _lib.load()
    n = counts.shape[0]
    G = int(d_grid.shape[1])
    if d_grid.shape[0] != n:
        raise ValueError("prob_t_pairs_grid: %d grid rows for %d branches" % (d_grid.shape[0], n))
    out = t.empty((n, G), dtype=t.float64, device=counts.device)
    mo = None
    if model_of is not None:
        mo = model_of if hasattr(model_of, "data_ptr") else _to_dev(np.asarray(model_of, np.int32), counts.device)
    check(lib.tt_prob_t_pairs_grid(q, n, _p(counts), _p(mo), C.byref(model.struct), _p(d_grid), G, _p(out),
                                   _stream()), "tt_prob_t_pairs_grid")
    return out


_MUT_WS = {}


def _mutation_workspace(dev, rows, P, n, threads_per_pattern, extra_bytes=0):
    """Device FP64 workspace of the counting kernels: `extra_bytes` (rounded
    up to 256) for the offset branch matrices, then one [rows][P] slice per
    chunk of branches, as many chunks (<= 64) as fill the GPU; cached per
    device and stream, grown when a call needs more."""
    t = torch()
    sms = _lib.load().tt_device_sm_count()
    want = max(1, min(64, n, -(-(sms * 2048) // max(1, P * threads_per_pattern))))
    need = want * rows * P + -(-extra_bytes // 256) * 32
    key = (str(dev), t.cuda.current_stream(dev).cuda_stream)
    buf = _MUT_WS.get(key)
    if buf is None or buf.numel() < need:
        buf = t.empty(max(need, 1), dtype=t.float64, device=dev)
        _MUT_WS[key] = buf
    return buf, int(buf.numel() * 8)


def mutation_counts(forest, model, p64, tree, d_node, pp, d_pp_row, pc, d_pc_row, precision):
    """Substitution counts of the 'marginal' GTR inference over the listed
    branches of one tree: (n_ija [q, q, P], T_ia [q, P]) device FP64
    (treetime/treeanc.py:1546-1563)."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    q = forest.q
    P = int(forest.trees_host["n_patterns"][tree])
    n = int(d_node.numel())
    n_ija = t.empty((q, q, P), dtype=t.float64, device=dev)
    T_ia = t.empty((q, P), dtype=t.float64, device=dev)
    ws, ws_bytes = _mutation_workspace(dev, q * q + q, P, n, 1 if q <= 5 else 32,
                                       extra_bytes=forest.n_nodes * (q * q + 1) * (4 if precision == "f32" else 8))
    check(lib.tt_mutation_counts(C.byref(forest.struct), C.byref(model.struct), int(tree), P, n, _p(d_node), _p(pp),
                                 _p(d_pp_row), _p(pc), _p(d_pc_row),
                                 _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64, _p(p64), _p(n_ija),
                                 _p(T_ia), _p(ws), ws_bytes, _stream()), "tt_mutation_counts")
    return n_ija, T_ia


def mutation_counts_ss(forest, gtr, bufs, d_node, pp, d_pp_row, pc, d_pc_row, precision):
    """mutation_counts under a GTR_site_specific model (one tree): every
    site's own P_a(t) (TreeTime's interpolated or exact expQt), FP64."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    q = forest.q
    P = int(forest.trees_host["n_patterns"][0])
    n = int(d_node.numel())
    arrs = _ss_model64(gtr, bufs, dev, need_stack=True)
    n_ija = t.empty((q, q, P), dtype=t.float64, device=dev)
    T_ia = t.empty((q, P), dtype=t.float64, device=dev)
    ws, ws_bytes = _mutation_workspace(dev, q * q + q, P, n, 1)
    check(lib.tt_mutation_counts_ss(C.byref(forest.struct), C.byref(arrs["struct"]), 0, P, n, _p(d_node), _p(pp),
                                    _p(d_pp_row), _p(pc), _p(d_pc_row),
                                    _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64, _p(n_ija),
                                    _p(T_ia), _p(ws), ws_bytes, _stream()), "tt_mutation_counts_ss")
    return n_ija, T_ia


def mutation_counts_joint(forest, tree, d_node, states, char_state, tips_use_states, tip_mismatch=None):
    """Substitution counts of the 'joint' GTR inference from the states of the
    last reconstruction: (n_ija [q, q, P], T_ia [q, P]) device FP64
    (treetime/treeanc.py:1564-1582)."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    q = forest.q
    P = int(forest.trees_host["n_patterns"][tree])
    n = int(d_node.numel())
    n_ija = t.empty((q, q, P), dtype=t.float64, device=dev)
    T_ia = t.empty((q, P), dtype=t.float64, device=dev)
    ws, ws_bytes = _mutation_workspace(dev, q * q + q, P, n, 1)
    cs = _to_dev(np.asarray(char_state, np.uint8), dev)
    mm = None if tip_mismatch is None else _to_dev(np.asarray(tip_mismatch, np.int32), dev)
    check(lib.tt_mutation_counts_joint(C.byref(forest.struct), int(tree), P, n, _p(d_node), _p(states), _p(cs),
                                       int(bool(tips_use_states)), _p(mm), _p(n_ija), _p(T_ia), _p(ws), ws_bytes,
                                       _stream()), "tt_mutation_counts_joint")
    return n_ija, T_ia


def branch_mutation_matrix(forest, model, p64, tree, node, pp, pp_row, pc, pc_row, precision):
    """[P, q, q] normalised joint distribution of the states at both ends of
    one branch (treetime/treeanc.py:1085-1120)."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    q = forest.q
    P = int(forest.trees_host["n_patterns"][tree])
    out = t.empty((P, q, q), dtype=t.float64, device=dev)
    d_node = _to_dev(np.array([node], np.int32), dev)
    d_pp = _to_dev(np.array([pp_row], np.int64), dev)
    d_pc = _to_dev(np.array([pc_row], np.int64), dev)
    check(lib.tt_branch_mutation_matrix(C.byref(forest.struct), C.byref(model.struct), int(tree), P, _p(d_node),
                                        _p(pp), _p(d_pp), _p(pc), _p(d_pc),
                                        _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64, _p(p64),
                                        _p(out), _stream()), "tt_branch_mutation_matrix")
    return out


def branch_mutation_matrix_ss(forest, gtr, bufs, node, pp, pp_row, pc, pc_row, precision):
    """branch_mutation_matrix under a GTR_site_specific model (one tree): every
    site's own P_a(t) (treetime/treeanc.py:1106-1108)."""
    t = torch()
    lib = _lib.load()
    dev = forest.device
    q = forest.q
    P = int(forest.trees_host["n_patterns"][0])
    arrs = _ss_model64(gtr, bufs, dev, need_stack=True)
    out = t.empty((P, q, q), dtype=t.float64, device=dev)
    d_node = _to_dev(np.array([node], np.int32), dev)
    d_pp = _to_dev(np.array([pp_row], np.int64), dev)
    d_pc = _to_dev(np.array([pc_row], np.int64), dev)
    check(lib.tt_branch_mutation_matrix_ss(C.byref(forest.struct), C.byref(arrs["struct"]), 0, P, _p(d_node),
                                           _p(pp), _p(d_pp), _p(pc), _p(d_pc),
                                           _lib.TT_PREC_F32 if precision == "f32" else _lib.TT_PREC_F64,
                                           _p(out), _stream()), "tt_branch_mutation_matrix_ss")
    return out


def _mini_forest(n_nodes, q, bl, device, mult=None, parent=None, n_int=None, P=1):
    """A one-tree forest struct for standalone per-branch calls."""
    dev = require_device(device)
    tr = np.zeros(1, dtype=[(n, np.int64) for n in ("node_base", "level_base", "pat_base", "tip_base", "prof_base",
                                                    "tipprof_base", "state_base")] +
                  [(n, np.int32) for n in ("n_int", "n_tip", "n_levels", "n_patterns", "model", "reserved")])
    tr[0] = (0, 0, 0, 0, 0, 0, 0, n_nodes if n_int is None else n_int, 0, 0, P, 0, 0)
    keep = {"trees": _to_dev(tr.view(np.uint8), dev), "bl": _to_dev(np.asarray(bl, np.float64), dev)}
    keep["parent"] = _to_dev(np.asarray(parent if parent is not None else np.full(n_nodes, -1), np.int32), dev)
    keep["mult"] = _to_dev(np.asarray(mult if mult is not None else np.ones(P), np.float64), dev)
    keep["tip_row"] = _to_dev(np.full(n_nodes, -1, np.int32), dev)
    w = WIDTHS[q]
    f = TTForest(1, q, w, 0, n_nodes, P, _p(keep["trees"]), None, None, None, _p(keep["parent"]), _p(keep["tip_row"]),
                 None, None, _p(keep["bl"]), None, _p(keep["mult"]), None, 0, 8, 0, 1, None, 0, 0, None, None, None, 1, 0)
    return f, keep


def expqt(gtr, t):
    """P(t) on the device; scalar t -> [q, q], array -> [n, q, q]."""
    if gtr.is_site_specific:
        return expqt_site_specific(gtr, t)
    tt = torch()
    scalar = np.ndim(t) == 0
    ts = np.atleast_1d(np.asarray(t, dtype=np.float64))
    check_exp(gtr, ts)
    model = model_for(gtr)
    q = gtr.n_states
    w = WIDTHS[q]
    f, keep = _mini_forest(len(ts), q, ts, model.device)
    p64 = tt.empty((len(ts), q, w), dtype=tt.float64, device=model.device)
    status = tt.zeros(1, dtype=tt.int32, device=model.device)
    check(_lib.load().tt_branch_pmats(C.byref(f), C.byref(model.struct), TTPmats(_p(p64), None, None, None),
                                      _p(status), _stream()), "tt_branch_pmats")
    _check_status(status)
    res = p64[:, :, :q].cpu().numpy()
    return res[0] if scalar else res


def expqt_site_specific(gtr, t):
    """[q, q, L] stack of per-site P(t) (interpolated when approximate) computed
    on the device with torch from the site eigendecompositions."""
    tt = torch()
    dev = require_device(None)
    lam, V, Vi = site_matrices(gtr)
    mu = np.asarray(gtr.mu, dtype=np.float64)
    Vd, Vid = _to_dev(V, dev), _to_dev(Vi, dev)

    def exact(x):
        e = tt.exp(_to_dev(lam * mu[:, None] * x, dev))
        return tt.einsum("aik,ak,akj->aij", Vd, e, Vid)

    if gtr.approximate and t * gtr.rate_scale < 10:
        grid = site_grid(gtr)
        hi = int(np.clip(np.searchsorted(grid, t), 1, len(grid) - 1))
        lo = hi - 1
        ylo, yhi = exact(grid[lo]), exact(grid[hi])
        res = (yhi - ylo) / (grid[hi] - grid[lo]) * (t - grid[lo]) + ylo
    else:
        res = exact(t)
    return res.permute(1, 2, 0).contiguous().cpu().numpy()


def propagate(gtr, profile, t, transpose=False, return_log=False):
    tt = torch()
    prof = np.asarray(profile, dtype=np.float64)
    if gtr.is_site_specific:
        dev = require_device(None)
        Qt = _to_dev(expqt_site_specific(gtr, t), dev)
        x = _to_dev(prof, dev)
        if transpose:
            res = tt.einsum("ai,jia->aj", x, Qt)
            return (tt.log(res) if return_log else res).cpu().numpy()
        res = tt.einsum("ai,ija->aj", x, Qt)
        return (tt.log(tt.clamp(res, min=ttconf.TINY_NUMBER)) if return_log else tt.clamp(res, min=0.0)).cpu().numpy()
    P = expqt(gtr, t)
    model = model_for(gtr)
    dev = model.device
    q = gtr.n_states
    d_prof = _to_dev(prof.reshape(-1, q), dev)
    d_p = _to_dev(np.ascontiguousarray(P), dev)
    res = tt.empty_like(d_prof)
    check(_lib.load().tt_propagate(q, d_prof.shape[0], _p(d_prof), _p(d_p), None, int(transpose), int(return_log),
                                   _p(res), _stream()), "tt_propagate")
    return res.cpu().numpy().reshape(prof.shape)


def pairs_to_counts(q, seq_pair, multiplicity):
    counts = np.zeros((q, q), dtype=np.float64)
    sp = np.asarray(seq_pair, dtype=np.int64).reshape(-1, 2)
    np.add.at(counts, (sp[:, 0], sp[:, 1]), np.asarray(multiplicity, dtype=np.float64))
    return counts


def state_pair(gtr, seq_p, seq_ch, pattern_multiplicity=None, ignore_gaps=False):
    """Histogram of (parent, child) state pairs on the device, returned in
    TreeTime's order and with its int cast (treetime/gtr.py:631-712)."""
    tt = torch()
    seq_p = np.asarray(seq_p)
    seq_ch = np.asarray(seq_ch)
    if seq_ch.shape != seq_p.shape:
        raise ValueError("GTR.state_pair: Sequence lengths do not match!")
    P = len(seq_p)
    mult = np.ones(P) if pattern_multiplicity is None else np.asarray(pattern_multiplicity, dtype=np.float64)
    q = gtr.n_states
    from .alphabets import chars_to_codes
    cs = char_state_table(gtr)
    sp, sc = cs[chars_to_codes(seq_p)], cs[chars_to_codes(seq_ch)]
    dev = require_device(None)
    f, keep = _mini_forest(2, q, np.zeros(2), dev, mult=mult, parent=[-1, 0], n_int=2, P=P)
    states = _to_dev(np.concatenate([sp, sc]).astype(np.uint8), dev)
    d_cs = _to_dev(cs, dev)
    hist = tt.zeros((2, q, q), dtype=tt.float64, device=dev)
    gap = gtr.gap_index
    check(_lib.load().tt_state_pairs(C.byref(f), _p(states), _p(d_cs), 1, -1 if gap is None else gap,
                                     int(bool(ignore_gaps)), None, _p(hist), _stream()), "tt_state_pairs")
    h = hist[1].cpu().numpy()
    if q < 10:
        order = [(i, j) for i in range(q) for j in range(q) if h[i, j]]
    else:
        codes = sp.astype(np.int64) * q + sc
        keep_mask = np.ones(P, dtype=bool)
        if ignore_gaps and gap is not None:
            keep_mask = (sp != gap) & (sc != gap)
        uniq, first = np.unique(codes[keep_mask], return_index=True)
        order = [divmod(int(c), q) for c in uniq[np.argsort(first, kind="stable")]]
    pairs = np.array(order, dtype=int).reshape(-1, 2)
    counts = np.array([h[i, j] for i, j in order], dtype=int)
    return pairs, counts


def prob_t_compressed(gtr, seq_pair, multiplicity, t, return_log=False):
    tt = torch()
    model = model_for(gtr)
    q = gtr.n_states
    counts = _to_dev(pairs_to_counts(q, seq_pair, multiplicity)[None], model.device)
    d_t = _to_dev(np.array([t], dtype=np.float64), model.device)
    out = tt.empty(1, dtype=tt.float64, device=model.device)
    check(_lib.load().tt_prob_t_pairs(q, 1, _p(counts), None, C.byref(model.struct), _p(d_t), _p(out), _stream()),
          "tt_prob_t_pairs")
    v = float(out.item())
    if t < 0:
        v = -ttconf.BIG_NUMBER
    return v if return_log else float(np.exp(v))


def prob_t_profiles(gtr, profile_pair, multiplicity, t, return_log=False, ignore_gaps=True):
    """Objective of the marginal branch-length mode, evaluated on the device with
    torch (treetime/gtr.py:922-963)."""
    tt = torch()
    if t < 0:
        v = -ttconf.BIG_NUMBER
    else:
        dev = require_device(None)
        Qt = _to_dev(np.asarray(expqt(gtr, t)), dev)
        pp, pc = (_to_dev(np.asarray(x, np.float64), dev) for x in profile_pair)
        m = _to_dev(np.asarray(multiplicity, np.float64), dev)
        if Qt.dim() == 3:
            res = tt.einsum("ai,ija,aj->a", pc, Qt, pp)
        else:
            res = tt.einsum("ai,ij,aj->a", pc, Qt, pp)
        term = m * tt.log(res + ttconf.SUPERTINY_NUMBER)
        if ignore_gaps and gtr.gap_index is not None:
            term = term * (1 - pp[:, gtr.gap_index]) * (1 - pc[:, gtr.gap_index])
        v = float(term.sum().item())
    return v if return_log else float(np.exp(v))


def optimal_t_compressed(gtr, seq_pair, multiplicity, profiles=False, tol=1e-10):
    model = model_for(gtr)
    q = gtr.n_states
    if not profiles:
        counts = _to_dev(pairs_to_counts(q, seq_pair, multiplicity)[None], model.device)
        tout, info = optimal_t_pairs(q, counts, model, tol=tol)
    else:
        pp, pc = (np.asarray(x, np.float64) for x in seq_pair)
        P = pp.shape[0]
        w = WIDTHS[q]
        dev = model.device
        f, keep = _mini_forest(2, q, np.zeros(2), dev, mult=multiplicity, parent=[-1, 0], n_int=2, P=P)
        pad = lambda a: np.pad(a, ((0, 0), (0, w - q)))
        d_pp = _to_dev(pad(pp), dev)
        d_pc = _to_dev(pad(pc), dev)
        tout, info = optimal_t_profiles(_ForestView(f, dev, q, P), model, [1], d_pp, [0], d_pc, [0], "f64",
                                        gtr.gap_index, True, tol)
    if int(info[0].item()) == -1:
        check(_lib.TT_ERR_BRACKET, "optimal_t_compressed")
    return float(tout[0].item())


class _ForestView:
    """The parts of a Forest the per-branch calls read: the C struct, the
    device, the alphabet size and the pattern count of its one tree."""

    def __init__(self, struct, device, q, n_patterns):
        self.struct = struct
        self.device = device
        self.q = q
        self.trees_host = np.array([(n_patterns,)], dtype=[("n_patterns", np.int32)])


# ----------------------------------------------------------------------------
# column compression on the device
# ----------------------------------------------------------------------------
def compress_columns(codes, ambiguous_code, device=None):
    """Pattern compression with the column classification on the device;
    identical output to seqdata.compress_codes."""
    tt = torch()
    dev = require_device(device)
    codes = np.ascontiguousarray(codes, dtype=np.uint8)
    n, L = codes.shape
    d = _to_dev(codes, dev)
    key = tt.empty(L, dtype=tt.int64, device=dev)
    fixed = tt.empty(L, dtype=tt.int32, device=dev)
    check(_lib.load().tt_compress_columns(_p(d), n, L, -1 if ambiguous_code is None else int(ambiguous_code),
                                          _p(key), _p(fixed), _stream()), "tt_compress_columns")
    key_h = key.cpu().numpy()
    fixed_h = fixed.cpu().numpy()
    uniq, first, inverse, counts = np.unique(key_h, return_index=True, return_inverse=True, return_counts=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    f2c = rank[inverse].astype(np.int64)
    mult = counts[order].astype(float)
    cols = first[order]
    # the pattern columns gathered on the device (one strided pass over the alignment)
    pc = d[:, _to_dev(cols.astype(np.int64), dev)].cpu().numpy()
    fx = fixed_h[cols]
    js = np.flatnonzero(fx >= 0)
    if len(js):
        sub = pc[:, js]
        hit = sub == ambiguous_code
        sub[hit] = np.broadcast_to(fx[js].astype(np.uint8), sub.shape)[hit]
        pc[:, js] = sub
    pos_sorted = np.argsort(f2c, kind="stable")
    bounds = np.concatenate(([0], np.cumsum(counts[order])))
    c2f = {p: pos_sorted[bounds[p]:bounds[p + 1]].astype(int) for p in range(len(order))}
    return pc, mult, f2c, c2f
