"""Named nucleotide substitution models.  Each builds pi and W and hands them to
``GTR.assign_rates``; the parameterisations (alphabets, which entries carry
kappa) are those of treetime/nuc_models.py so that a model name means the
same rate matrix in both code bases."""

import numpy as np

from .alphabets import alphabets
from .gtr import GTR


def _alphabet_size(alphabet):
    if isinstance(alphabet, str) and alphabet in alphabets:
        return len(alphabets[alphabet])
    return len(np.array(alphabet))


def _transition_W(kappa):
    """A,C,G,T rate matrix with kappa on the transitions A<->G and C<->T."""
    W = np.ones((4, 4))
    W[0, 2] = W[2, 0] = W[1, 3] = W[3, 1] = kappa
    return W


def JC69(mu=1.0, alphabet="nuc", **kwargs):
    n = _alphabet_size(alphabet)
    gtr = GTR(alphabet=alphabet)
    gtr.assign_rates(mu=mu, pi=np.ones(n), W=np.ones((n, n)))
    return gtr


def K80(mu=1.0, kappa=0.1, **kwargs):
    gtr = GTR(alphabet="nuc_nogap")
    gtr.assign_rates(mu=mu, pi=np.full(4, 0.25), W=_transition_W(kappa))
    return gtr


def F81(mu=1.0, pi=None, alphabet="nuc", **kwargs):
    pi = np.full(4, 0.25) if pi is None else np.array(pi, dtype=float)
    n = _alphabet_size(alphabet)
    if n != len(pi):
        pi = np.ones(n)
    gtr = GTR(alphabet=alphabet)
    gtr.assign_rates(mu=mu, pi=pi / pi.sum(), W=np.ones((n, n)))
    return gtr


def HKY85(mu=1.0, pi=None, kappa=0.1, **kwargs):
    pi = np.full(4, 0.25) if pi is None else np.array(pi, dtype=float)
    if len(pi) != 4:
        pi = np.ones(4)
    gtr = GTR(alphabet="nuc_nogap")
    gtr.assign_rates(mu=mu, pi=pi / pi.sum(), W=_transition_W(kappa))
    return gtr


def T92(mu=1.0, pi_GC=0.5, kappa=0.1, **kwargs):
    if pi_GC >= 1.0:
        raise ValueError("The relative GC content specified is larger than 1.0!")
    pi = np.array([(1.0 - pi_GC) * 0.5, pi_GC * 0.5, pi_GC * 0.5, (1.0 - pi_GC) * 0.5])
    gtr = GTR(alphabet="nuc_nogap")
    gtr.assign_rates(mu=mu, pi=pi, W=_transition_W(kappa))
    return gtr


def TN93(mu=1.0, kappa1=1.0, kappa2=1.0, pi=None, **kwargs):
    pi = np.full(4, 0.25) if pi is None else np.array(pi, dtype=float)
    W = np.array([[1, kappa1, 1, kappa1], [kappa1, 1, kappa1, kappa2],
                  [1, kappa1, 1, kappa1], [kappa1, kappa2, kappa1, 1]], dtype=float)
    pi = pi / pi.sum()
    if len(pi) != 4:
        pi = np.ones(4)
    # TreeTime builds TN93 on the 5-letter 'nuc' alphabet, where the 4-state
    # pi and W do not fit and defaults are used; kept for equal results.
    gtr = GTR(alphabet="nuc")
    gtr.assign_rates(mu=mu, pi=pi, W=W)
    return gtr
