"""General-time-reversible substitution models (host side).

The model set-up is host work in FP64, as in TreeTime: normalisation of the
rate matrix and the symmetrised eigendecomposition (treetime/gtr.py:235-283,
:612-629; treetime/gtr_site_specific.py:43-114, :312-348).  Everything that
runs per branch or per alignment pattern -- P(t) = V·exp(Λt)·V⁻¹, profile
propagation, the pair likelihood and the branch-length optimiser -- runs on
the GPU through ``treetime_gb300.engine``; the methods here with the same
names as TreeTime's (``expQt``, ``propagate_profile``, ``evolve``,
``prob_t_compressed``, ``prob_t_profiles``, ``optimal_t_compressed``,
``state_pair``) are thin device calls.
"""

import numpy as np

from . import config as ttconf
from .alphabets import alphabets, alphabet_synonyms, fresh_profile_map
from .errors import MissingDataError


def avg_transition(W, pi, gap_index=None):
    """Average substitution rate pi·W·pi, excluding transitions into the gap
    state when the alphabet has one (treetime/gtr.py:7-11)."""
    total = np.einsum("i,ij,j", pi, W, pi)
    if gap_index is None:
        return total
    return (total - np.sum(pi * W[:, gap_index]) * pi[gap_index]) / (1 - pi[gap_index])


def eig_single_site(W, p):
    """Eigendecomposition of the rate matrix through its symmetrised form
    sqrt(pi)·W·sqrt(pi) with diagonal -sum_j W_ij pi_j; eigenvectors are
    rescaled by their 1-norm so that V·V⁻¹ = I (treetime/gtr.py:612-629).
    Returns (eigenvalues, V, V⁻¹)."""
    if abs(np.diag(W).sum()) >= 1e-10:
        raise ValueError("rate matrix W must have a zero diagonal")
    sq = np.sqrt(p)
    sym = W * np.outer(sq, sq)
    np.fill_diagonal(sym, -np.sum(W * p, axis=1))
    lam, vec = np.linalg.eigh(sym)
    right = vec.T * sq
    norm1 = np.sum(np.abs(right), axis=1)
    return lam, right.T / norm1, (vec * norm1).T / sq


class GTR:
    """Reversible substitution model with a single rate matrix."""

    def __init__(self, alphabet="nuc", prof_map=None, logger=None):
        self.debug = False
        self.is_site_specific = False
        if isinstance(alphabet, str):
            if alphabet not in alphabet_synonyms:
                raise AttributeError("Unknown alphabet type specified")
            name = alphabet_synonyms[alphabet]
            self.alphabet = alphabets[name].copy()
            self.profile_map = fresh_profile_map(name)
        else:
            self.alphabet = np.array(alphabet)
            if prof_map is None:
                self.profile_map = {s: x for s, x in zip(self.alphabet.tolist(), np.eye(len(self.alphabet)))}
            else:
                self.profile_map = {k: np.asarray(v, dtype=float) for k, v in prof_map.items()}
        self.state_index = {s: i for i, s in enumerate(self.alphabet.tolist())}
        self.logger = logger if logger is not None else (lambda *a, **k: None)
        self.n_states = len(self.alphabet)
        self._find_gap_and_ambiguous()
        self.v = self.v_inv = self.eigenvals = None
        self._device_cache = None
        self.assign_rates()

    def _find_gap_and_ambiguous(self):
        n = len(self.alphabet)
        amb = [c for c, x in self.profile_map.items() if np.asarray(x).sum() == n]
        self.ambiguous = ("N" if "N" in amb else amb[0]) if amb else None
        self.gap_index = self.state_index.get("-")

    # ---------------------------------------------------------------- rates
    @property
    def mu(self):
        return self._mu

    @mu.setter
    def mu(self, value):
        self.assign_rates(mu=value, pi=self.Pi, W=self.W)

    @property
    def Pi(self):
        return self._Pi

    @Pi.setter
    def Pi(self, value):
        self.assign_rates(mu=self.mu, pi=value, W=self.W)

    @property
    def W(self):
        return self._W

    @W.setter
    def W(self, value):
        self.assign_rates(mu=self.mu, pi=self.Pi, W=value)

    @property
    def Q(self):
        Q = (self.W * self.Pi).T
        np.fill_diagonal(Q, -np.sum(Q, axis=0))
        return Q

    def assign_rates(self, mu=1.0, pi=None, W=None):
        """Set mu, pi and W.  pi is normalised to one; W loses its diagonal and
        is scaled so that the average rate is one, the scale moving into mu
        (treetime/gtr.py:235-283).  As in TreeTime, the stored W is the input
        W (not its symmetrised copy)."""
        n = len(self.alphabet)
        self._mu = mu
        self.is_site_specific = False
        if pi is not None and len(pi) == n:
            Pi = np.array(pi, dtype=float)
        else:
            if pi is not None:
                self.logger("length of equilibrium frequency vector does not match alphabet length", 4, warn=True)
            Pi = np.ones(n)
        self._Pi = Pi / np.sum(Pi)
        if W is None or np.shape(W) != (n, n):
            if W is not None:
                self.logger("Substitution matrix size does not match alphabet size", 4, warn=True)
            W = np.ones((n, n))
            np.fill_diagonal(W, 0.0)
            np.fill_diagonal(W, -W.sum(axis=0))
        else:
            W = np.array(W, dtype=float)
        np.fill_diagonal(W, 0)
        rate = avg_transition(W, self._Pi, gap_index=self.gap_index)
        self._W = W / rate
        self._mu *= rate
        self._eig()

    def _eig(self):
        self.eigenvals, self.v, self.v_inv = eig_single_site(self._W, self._Pi)
        self._device_cache = None

    def average_rate(self):
        return self.mu * avg_transition(self.W, self.Pi, gap_index=self.gap_index)

    @classmethod
    def custom(cls, mu=1.0, pi=None, W=None, **kwargs):
        gtr = cls(**kwargs)
        gtr.assign_rates(mu=mu, pi=pi, W=W)
        return gtr

    @classmethod
    def infer(cls, nij, Ti, root_state, fixed_pi=None, pc=1.0, gap_limit=0.01, **kwargs):
        """Fit mu, pi and W to substitution counts n_ij (i derived, j ancestral),
        times T_i spent in each state and root state counts by TreeTime's fixed
        point iteration of n_ij + pc = pi_i W_ij (T_j + pc + root_state)
        (treetime/gtr.py:492-599): at most 40 rounds until |pi - pi_old| <= 1e-5,
        then the gap frequency set to gap_limit.  Host work on q x q arrays; the
        counts come from the GPU (TreeAnc.infer_gtr)."""
        gtr = cls(**kwargs)
        gtr.logger("GTR: model inference ", 1)
        dp, n_iter_max = 1e-5, 40
        nij = np.array(nij, dtype=float)
        Ti = np.asarray(Ti, dtype=float)
        pc_mat = pc * np.ones_like(nij)
        np.fill_diagonal(pc_mat, 0.0)
        np.fill_diagonal(nij, 0.0)
        count = 0
        pi_old = np.zeros_like(Ti)
        pi = np.ones_like(Ti) if fixed_pi is None else np.copy(fixed_pi)
        pi /= pi.sum()
        W_ij = np.ones_like(nij)
        mu = (nij.sum() + pc) / (Ti.sum() + pc)
        while np.linalg.norm(pi_old - pi) > dp and count < n_iter_max:
            gtr.logger(" ".join(map(str, ["GTR inference iteration", count, "change:",
                                          np.linalg.norm(pi_old - pi)])), 3)
            count += 1
            pi_old = np.copy(pi)
            W_ij = ((nij + nij.T + 2 * pc_mat) / mu
                    / (np.outer(pi, Ti) + np.outer(Ti, pi) + ttconf.TINY_NUMBER + 2 * pc_mat))
            np.fill_diagonal(W_ij, 0)
            W_ij = W_ij / avg_transition(W_ij, pi, gap_index=gtr.gap_index)
            if fixed_pi is None:
                pi = (np.sum(nij + pc_mat, axis=1) + root_state) / (
                    ttconf.TINY_NUMBER + mu * np.dot(W_ij, Ti) + root_state.sum() + np.sum(pc_mat, axis=1))
                pi /= pi.sum()
                mu = (nij.sum() + pc) / (np.sum(pi * (W_ij.dot(Ti))) + pc)
            else:
                mu = (nij.sum() + pc) / (np.sum(pi * (W_ij.dot(pi))) * Ti.sum() + pc)
        if count >= n_iter_max:
            gtr.logger("WARNING: maximum number of iterations has been reached in GTR inference", 3, warn=True)
            if np.linalg.norm(pi_old - pi) > dp:
                gtr.logger("the iterative scheme has not converged", 3, warn=True)
            elif np.abs(1 - np.max(pi.sum(axis=0))) > dp:
                gtr.logger("the iterative scheme has converged, but proper normalization was not reached", 3,
                           warn=True)
        if gtr.gap_index is not None:
            if pi[gtr.gap_index] < gap_limit:
                gtr.logger("The model allows for gaps which are estimated to occur at a low fraction of %1.3e"
                           % pi[gtr.gap_index] + " this can potentially result in artificats."
                           + " gap fraction will be set to %1.4f" % gap_limit, 2, warn=True)
            pi[gtr.gap_index] = gap_limit
            pi /= pi.sum()
        gtr.assign_rates(mu=mu, W=W_ij, pi=pi)
        return gtr

    @classmethod
    def random(cls, mu=1.0, alphabet="nuc", rng=None):
        """Random model: pi and W uniform on [0,1) from ``rng`` in the order
        pi then W (treetime/gtr.py:463-489)."""
        rng = np.random.default_rng() if rng is None else rng
        gtr = cls(alphabet)
        n = gtr.alphabet.shape[0]
        pi = 1.0 * rng.random(size=n)
        W = 1.0 * rng.random(size=(n, n))
        gtr.assign_rates(mu=mu, pi=pi, W=W)
        return gtr

    @staticmethod
    def standard(model, **kwargs):
        """Named nucleotide models: JC69, K80, F81, HKY85, T92, TN93
        (treetime/gtr.py:318-461, treetime/nuc_models.py)."""
        from .nuc_models import JC69, K80, F81, HKY85, T92, TN93
        m = model.lower()
        if m in ["jc", "jc69", "jukes-cantor", "jukes-cantor69", "jukescantor", "jukescantor69"]:
            gtr = JC69(**kwargs)
        elif m in ["k80", "kimura80", "kimura1980"]:
            gtr = K80(**kwargs)
        elif m in ["f81", "felsenstein81", "felsenstein1981"]:
            gtr = F81(**kwargs)
        elif m in ["hky", "hky85", "hky1985"]:
            gtr = HKY85(**kwargs)
        elif m in ["t92", "tamura92", "tamura1992"]:
            gtr = T92(**kwargs)
        elif m in ["tn93", "tamura_nei_93", "tamuranei93"]:
            gtr = TN93(**kwargs)
        else:
            raise KeyError("The GTR model '{}' is not in the list of available models.".format(model))
        gtr.mu = kwargs["mu"] if "mu" in kwargs else 1.0
        return gtr

    # ------------------------------------------------------ host-side checks
    def check_branch_lengths(self, t):
        """exp(mu·lambda·t) must not blow up: TreeTime raises ValueError when
        any mu·lambda·t exceeds 10 (treetime/gtr.py:1042-1047)."""
        t = np.asarray(t, dtype=float)
        if t.size == 0:
            return
        lam = np.asarray(self.eigenvals)
        mu = np.asarray(self.mu)
        top = np.max(mu * lam) if lam.ndim == 1 else np.max(mu[None, :] * lam)
        if top * (np.max(t) if top > 0 else np.min(t)) > 10:
            raise ValueError(
                "Error in computing exp(Q * t): Q has positive eigenvalues or the branch length t is too large. "
                "This is most likely caused by incorrect input data."
            )

    # --------------------------------------------------------- device calls
    def device_model(self, device=None):
        """Cached FP64 device copies of V, V⁻¹, eigenvalues, pi and the profile table."""
        from . import engine
        return engine.model_for(self, device)

    def expQt(self, t):
        """P(t) = max(0, V·diag(exp(mu·lambda·t))·V⁻¹) on the GPU; ``t`` may be a
        scalar (returns q×q) or an array (returns len(t)×q×q)."""
        from . import engine
        return engine.expqt(self, t)

    def expQs(self, s):
        return self.expQt(s ** 2)

    def propagate_profile(self, profile, t, return_log=False):
        """Child -> parent message ``profile·P(t)`` (log if requested), on the GPU
        (treetime/gtr.py:965-995)."""
        from . import engine
        return engine.propagate(self, profile, t, transpose=False, return_log=return_log)

    def evolve(self, profile, t, return_log=False):
        """Parent -> child message ``profile·P(t)ᵀ`` on the GPU
        (treetime/gtr.py:997-1025)."""
        from . import engine
        return engine.propagate(self, profile, t, transpose=True, return_log=return_log)

    def state_pair(self, seq_p, seq_ch, pattern_multiplicity=None, ignore_gaps=False):
        """(parent, child) state-pair histogram weighted by pattern
        multiplicity, on the GPU (treetime/gtr.py:631-712)."""
        from . import engine
        return engine.state_pair(self, seq_p, seq_ch, pattern_multiplicity, ignore_gaps)

    def prob_t_compressed(self, seq_pair, multiplicity, t, return_log=False):
        from . import engine
        return engine.prob_t_compressed(self, seq_pair, multiplicity, t, return_log)

    def prob_t(self, seq_p, seq_ch, t, pattern_multiplicity=None, return_log=False, ignore_gaps=True):
        pairs, mult = self.state_pair(seq_p, seq_ch, pattern_multiplicity=pattern_multiplicity, ignore_gaps=ignore_gaps)
        return self.prob_t_compressed(pairs, mult, t, return_log=return_log)

    def prob_t_profiles(self, profile_pair, multiplicity, t, return_log=False, ignore_gaps=True):
        from . import engine
        return engine.prob_t_profiles(self, profile_pair, multiplicity, t, return_log, ignore_gaps)

    def optimal_t(self, seq_p, seq_ch, pattern_multiplicity=None, ignore_gaps=False):
        pairs, mult = self.state_pair(seq_p, seq_ch, pattern_multiplicity=pattern_multiplicity, ignore_gaps=ignore_gaps)
        return self.optimal_t_compressed(pairs, mult)

    def optimal_t_compressed(self, seq_pair, multiplicity, profiles=False, tol=1e-10):
        """Branch length maximising the pair likelihood (Brent in s = sqrt(t)),
        on the GPU (treetime/gtr.py:816-920)."""
        from . import engine
        return engine.optimal_t_compressed(self, seq_pair, multiplicity, profiles=profiles, tol=tol)

    def sequence_logLH(self, seq, pattern_multiplicity=None):
        if pattern_multiplicity is None:
            pattern_multiplicity = np.ones_like(seq, dtype=float)
        return float(sum(np.sum((seq == s) * pattern_multiplicity * np.log(self.Pi[i]))
                         for i, s in enumerate(self.alphabet)))

    def __str__(self):
        lines = ["Substitution rate (mu): %s" % np.round(self.mu, 6), "", "Equilibrium frequencies (pi_i):"]
        for a, p in zip(self.alphabet, self.Pi):
            lines.append("  %s: %s" % (a, np.round(p, 4)))
        return "\n".join(lines) + "\n"


class GTR_site_specific(GTR):
    """Per-site equilibrium frequencies and rates with a shared W
    (treetime/gtr_site_specific.py).  ``approximate=True`` evaluates P(t) by
    linear interpolation on the 62-point time grid that TreeTime uses; the
    device code reproduces it in the eigenbasis, because interpolating the
    matrices V·diag(e^{mu·lambda·t_k})·V⁻¹ linearly in t equals
    V·diag(interpolated e)·V⁻¹."""

    def __init__(self, seq_len=1, approximate=True, **kwargs):
        self.seq_len = seq_len
        self.approximate = approximate
        super().__init__(**kwargs)
        self.is_site_specific = True

    @property
    def Q(self):
        tmp = np.einsum("ia,ij->ija", self.Pi, self.W)
        diag = np.sum(tmp, axis=0)
        for x in range(tmp.shape[-1]):
            np.fill_diagonal(tmp[:, :, x], -diag[:, x])
        return tmp

    def assign_rates(self, mu=1.0, pi=None, W=None):
        """Per-site pi (q×L) and mu (L), shared W normalised by the mean rate
        over sites (treetime/gtr_site_specific.py:43-114)."""
        if not np.isscalar(mu) and pi is not None and len(np.shape(pi)) == 2:
            if np.shape(mu)[0] != np.shape(pi)[1]:
                raise ValueError(
                    "GTR_site_specific: length of rate vector (got {}) and equilibrium frequency vector (got {}) must match!".format(
                        np.shape(mu)[0], np.shape(pi)[1]))
        n = len(self.alphabet)
        if np.isscalar(mu):
            self._mu = mu * np.ones(self.seq_len)
        else:
            self._mu = np.array(mu, dtype=float)
            self.seq_len = self._mu.shape[0]
        if pi is not None and np.shape(pi)[0] == n and len(np.shape(pi)) == 2:
            self.seq_len = np.shape(pi)[1]
            Pi = np.array(pi, dtype=float)
        elif pi is not None:
            if len(pi) == n:
                Pi = np.repeat([pi], self.seq_len, axis=0).T
            else:
                raise ValueError(
                    "GTR_site_specific: length of equilibrium frequency vector (got {}) does not match alphabet length {}".format(
                        len(pi), n))
        else:
            Pi = np.ones((n, self.seq_len))
        self._Pi = Pi / np.sum(Pi, axis=0)
        if W is None or np.shape(W) != (n, n):
            if W is not None:
                raise ValueError(
                    "GTR_site_specific: Size of substitution matrix (got {}) does not match alphabet length {}".format(
                        np.shape(W), n))
            W = np.ones((n, n))
            np.fill_diagonal(W, 0.0)
            np.fill_diagonal(W, -W.sum(axis=0))
        else:
            W = 0.5 * (np.array(W, dtype=float) + np.array(W, dtype=float).T)
        np.fill_diagonal(W, 0)
        rate = np.einsum("ia,ij,ja", self._Pi, W, self._Pi) / self.seq_len
        self._W = W / rate
        self._mu *= rate
        self.is_site_specific = True
        self._eig()
        self._make_time_grid()

    def _eig(self):
        lam, vec, vinv = [], [], []
        W = self._W
        np.fill_diagonal(W, 0)
        for a in range(self.seq_len):
            ev, v, vi = eig_single_site(W, self._Pi[:, a])
            lam.append(ev)
            vec.append(v)
            vinv.append(vi)
        # TreeTime's layouts: eigenvals [q, L], v and v_inv [q, q, L] with
        # v[j, i, a] = V_a[i, j] and v_inv[k, j, a] = V⁻¹_a[j, k]
        self.eigenvals = np.array(lam).T
        self.v = np.swapaxes(np.array(vec), 0, -1)
        self.v_inv = np.swapaxes(np.array(vinv), 0, -1)
        self._device_cache = None

    def site_matrices(self):
        """(lambda [L, q], V [L, q, q], V⁻¹ [L, q, q]) with V_a[i, j] row-major."""
        lam = np.ascontiguousarray(self.eigenvals.T)
        V = np.ascontiguousarray(np.transpose(self.v, (2, 1, 0)))
        Vi = np.ascontiguousarray(np.transpose(self.v_inv, (2, 1, 0)))
        return lam, V, Vi

    def _make_time_grid(self):
        """Time grid of the linear expQt interpolation
        (treetime/gtr_site_specific.py:331-348)."""
        self.rate_scale = self.average_rate().mean()
        self.t_grid = (1.0 / self.rate_scale) * np.concatenate((
            np.linspace(0, 0.1, 11)[:-1],
            np.linspace(0.1, 1, 21)[:-1],
            np.linspace(1, 5, 21)[:-1],
            np.linspace(5, 10, 11),
        ))

    def average_rate(self):
        if self.Pi.shape[1] > 1:
            return np.einsum("a,ia,ij,ja->a", self.mu, self.Pi, self.W, self.Pi)
        return self.mu * np.einsum("ia,ij,ja->a", self.Pi, self.W, self.Pi)

    @classmethod
    def infer(cls, sub_ija, T_ia, root_state, pc=1.0, gap_limit=0.01, Nit=30, dp=1e-5, **kwargs):
        """Per-site fit of pi_ia and mu_a with a shared W to per-site counts
        n_ija and times T_ia (treetime/gtr_site_specific.py:208-310): at most
        Nit rounds of the fixed point iteration until |p - p_old| <= dp, gap
        frequencies set to gap_limit per site.  Host work; the counts come from
        the GPU (TreeAnc.infer_gtr)."""
        gtr = cls(**kwargs)
        gtr.logger("GTR: model inference ", 1)
        q = len(gtr.alphabet)
        L = sub_ija.shape[-1]
        n_iter = 0
        n_ija = np.copy(sub_ija)
        n_ija[range(q), range(q), :] = 0
        n_ij = n_ija.sum(axis=-1)
        m_ia = np.sum(n_ija, axis=1) + root_state + pc
        n_a = n_ija.sum(axis=1).sum(axis=0) + pc
        Lambda = np.sum(root_state, axis=0) + q * pc
        p_ia_old = np.zeros((q, L))
        p_ia = np.ones((q, L)) / q
        mu_a = np.ones(L)
        W_ij = np.ones((q, q)) - np.eye(q)
        while (np.linalg.norm(p_ia_old - p_ia) > dp) and n_iter < Nit:
            gtr.logger(" ".join(map(str, ["GTR inference iteration", n_iter, "change:",
                                          np.linalg.norm(p_ia_old - p_ia)])), 3)
            n_iter += 1
            p_ia_old = np.copy(p_ia)
            S_ij = np.einsum("a,ia,ja", mu_a, p_ia, T_ia)
            W_ij = (n_ij + n_ij.T + pc) / (S_ij + S_ij.T + pc)
            avg_pi = p_ia.mean(axis=-1)
            average_rate = W_ij.dot(avg_pi).dot(avg_pi)
            W_ij = W_ij / average_rate
            mu_a *= average_rate
            p_ia = m_ia / (mu_a * np.dot(W_ij, T_ia) + Lambda)
            p_ia = p_ia / p_ia.sum(axis=0)
            mu_a = n_a / (pc + np.einsum("ia,ij,ja->a", p_ia, W_ij, T_ia))
        if n_iter >= Nit:
            gtr.logger("WARNING: maximum number of iterations has been reached in GTR inference", 3, warn=True)
            if np.linalg.norm(p_ia_old - p_ia) > dp:
                gtr.logger("the iterative scheme has not converged", 3, warn=True)
        if gtr.gap_index is not None:
            for p in range(p_ia.shape[-1]):
                if p_ia[gtr.gap_index, p] < gap_limit:
                    gtr.logger("The model allows for gaps which are estimated to occur at a low fraction of %1.3e"
                               % p_ia[gtr.gap_index, p] + "\n\t\tthis can potentially result in artifacts."
                               + "\n\t\tgap fraction will be set to %1.4f" % gap_limit, 4, warn=True)
                p_ia[gtr.gap_index, p] = gap_limit
                p_ia[:, p] /= p_ia[:, p].sum()
        gtr.assign_rates(mu=mu_a, W=W_ij, pi=p_ia)
        return gtr

    @classmethod
    def random(cls, L=1, avg_mu=1.0, alphabet="nuc", pi_dirichlet_alpha=1, W_dirichlet_alpha=3.0,
               mu_gamma_alpha=3.0, rng=None):
        """Random site-specific model, draws in TreeTime's order
        (treetime/gtr_site_specific.py:117-171)."""
        rng = np.random.default_rng() if rng is None else rng
        gtr = cls(alphabet=alphabets[alphabet], seq_len=L)
        n = gtr.alphabet.shape[0]
        pi = 1.0 * rng.gamma(pi_dirichlet_alpha, size=(n, L)) if pi_dirichlet_alpha else np.ones((n, L))
        pi /= pi.sum(axis=0)
        tmp = 1.0 * rng.gamma(W_dirichlet_alpha, size=(n, n)) if W_dirichlet_alpha else np.ones((n, n))
        tmp = np.tril(tmp, k=-1)
        W = tmp + tmp.T
        mu = rng.gamma(mu_gamma_alpha, size=(L,)) if mu_gamma_alpha else np.ones(L)
        gtr.assign_rates(mu=mu, pi=pi, W=W)
        gtr.mu = gtr.mu * (avg_mu / np.mean(gtr.average_rate()))
        return gtr

    def check_branch_lengths(self, t):
        t = np.asarray(t, dtype=float)
        if t.size == 0:
            return
        # only the exact path raises in TreeTime; the interpolated one cannot
        top = np.max(self.mu[None, :] * self.eigenvals)
        if top > 0 and top * np.max(t) > 10:
            raise ValueError(
                "Error in computing exp(Q * t): Q has positive eigenvalues or the branch length t is too large.")
