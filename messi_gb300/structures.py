"""Host-side structure utilities (no GPU): the KH99 prior of a structure.

calculateKH99prior restates src/InsideOutsideAlgorithm.jl:86-144: the
structure is parsed top-down with the unfolded KH99 rules (S -> sS | dFdS | s
| dFd, F -> dFd | sS | dFdS, L -> s | dFd) and the log-probabilities of the
rules used are summed.  ``paired`` uses the reference's convention: 1-based
partner per column, 0 when unpaired.
"""
import math

import numpy as np

_P = dict(LS=0.868534, S_s=0.117609877998, S_dFd=0.013856122002, F_dFd=0.787640, F_LS=0.21236, L_s=0.894603,
          L_dFd=0.105397)
# (symbol, right-hand side) -> log-probability of the unfolded rule
_RULES = {
    ("S", "sS"): math.log(_P["LS"] * _P["L_s"]),
    ("S", "dFdS"): math.log(_P["LS"] * _P["L_dFd"]),
    ("S", "s"): math.log(_P["S_s"]),
    ("S", "dFd"): math.log(_P["S_dFd"]),
    ("F", "dFd"): math.log(_P["F_dFd"]),
    ("F", "sS"): math.log(_P["F_LS"] * _P["L_s"]),
    ("F", "dFdS"): math.log(_P["F_LS"] * _P["L_dFd"]),
    ("L", "s"): math.log(_P["L_s"]),
    ("L", "dFd"): math.log(_P["L_dFd"]),
}


def calculateKH99prior(pairedsites):
    """Log prior of one structure (1-based partners, 0 = unpaired).  Spans
    no rule derives add nothing, as in the reference's parse loop."""
    paired = np.asarray(pairedsites, dtype=np.int64)
    L = len(paired)
    if L == 0:
        return 0.0
    ll = 0.0
    stack = [("S", 1, L)]
    while stack:
        sym, s, e = stack.pop()
        k = int(paired[s - 1])
        if k == 0:
            if s == e and (sym, "s") in _RULES:
                ll += _RULES[(sym, "s")]
            elif s < e and (sym, "sS") in _RULES:
                ll += _RULES[(sym, "sS")]
                stack.append(("S", s + 1, e))
        elif k > s:
            if k == e and (sym, "dFd") in _RULES:
                ll += _RULES[(sym, "dFd")]
                stack.append(("F", s + 1, k - 1))
            elif k != e and (sym, "dFdS") in _RULES:
                ll += _RULES[(sym, "dFdS")]
                stack.append(("F", s + 1, k - 1))
                stack.append(("S", k + 1, e))
    return ll
