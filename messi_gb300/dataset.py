"""Alignment + tree ingest, mirroring MESSI's ``Dataset``.

Host-side mirror of:
  * src/AlignmentIO.jl:18-48  ``getalignmentfromfastaandnewick`` (FASTA + Newick)
  * src/Tree.jl:114-171       Newick parsing (``gettreefromnewick``)
  * src/Tree.jl:45-55         ``roottree`` (splits the first child's branch)
  * src/Tree.jl:190-208       ``annotatetree`` / ``getnodelist`` (pre-order numbering)
  * src/Dataset.jl:13-96      IUPAC -> 4-bit nucleotide masks (gap = all four)
  * src/Dataset.jl:121-198    ``Dataset`` (gap frequencies, observed frequencies)

The per-node column-pattern compression (``subcolumnrefs``,
src/Dataset.jl:180-196) is done inside the GPU library when a dataset handle
is created.

Nucleotide masks: bit 0 = A, bit 1 = C, bit 2 = G, bit 3 = U/T; 15 = gap.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# src/Dataset.jl:13-96 (setnucleotides), as 4-bit masks
IUPAC_MASK = {
    "A": 1, "C": 2, "G": 4, "T": 8, "U": 8,
    "B": 2 | 4 | 8, "D": 1 | 4 | 8, "H": 1 | 2 | 8, "K": 4 | 8, "M": 1 | 2, "R": 1 | 4,
    "S": 2 | 4, "V": 1 | 2 | 4, "W": 1 | 8, "Y": 2 | 8,
}
NUCMAPPING = {"A": 0, "C": 1, "G": 2, "T": 3, "U": 3}  # src/Dataset.jl:6


def char_mask(c: str) -> int:
    return IUPAC_MASK.get(c.upper(), 15)


_MASK_LUT = np.array([char_mask(chr(b)) for b in range(256)], dtype=np.uint8)
_NUC_LUT = np.array([NUCMAPPING.get(chr(b), -1) for b in range(256)], dtype=np.int8)


class TreeNode:
    """src/Tree.jl:20-30."""

    def __init__(self, branchlength=0.0, name=""):
        self.parent: Optional["TreeNode"] = None
        self.children: List["TreeNode"] = []
        self.branchlength = float(branchlength)
        self.name = name
        self.nodeindex = 0
        self.seqindex = 0

    def addchild(self, child):
        child.parent = self
        self.children.append(child)

    def isleaf(self):
        return len(self.children) == 0


def _split_top(s):
    parts, depth, cur = [], 0, []
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    if cur:
        parts.append("".join(cur))
    return parts


def parse_newick(newick: str) -> TreeNode:
    """src/Tree.jl:114-171: children inside the outermost parentheses, then
    ``name:branchlength``."""
    s = newick.strip().rstrip(";").strip()
    close = s.rfind(")")
    childstrings = []
    tag = s
    if close >= 0:
        tag = s[close + 1:]
        childstrings = _split_top(s[1:close])
    spl = tag.split(":")
    name = spl[0].strip() if spl else ""
    bl = float(spl[1]) if len(spl) > 1 and spl[1].strip() else 0.0
    node = TreeNode(bl, name)
    for cs in childstrings:
        node.addchild(parse_newick(cs))
    return node


def to_newick(node: TreeNode) -> str:
    def rec(n):
        if n.isleaf():
            return f"{n.name}:{n.branchlength!r}"
        return "(" + ",".join(rec(c) for c in n.children) + f"){n.name}:{n.branchlength!r}"

    return rec(node) + ";"


def roottree(root: TreeNode, index: int = 0) -> TreeNode:
    """src/Tree.jl:45-55: new root above the `index`-th child, its branch split in half."""
    newroot = TreeNode(0.0, "")
    child = root.children.pop(index)
    child.parent = None
    newroot.addchild(child)
    br = child.branchlength / 2.0
    child.branchlength = br
    root.branchlength = br
    root.parent = None
    newroot.addchild(root)
    return newroot


def getnodelist(node: TreeNode, out=None):
    """Pre-order node list (src/Tree.jl:202-208)."""
    if out is None:
        out = []
    stack = [node]
    while stack:
        n = stack.pop()
        out.append(n)
        stack.extend(reversed(n.children))
    return out


def parse_fasta(text: str):
    names, seqs, cur = [], [], None
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            names.append(line[1:].strip())
            seqs.append([])
            cur = seqs[-1]
        elif cur is not None:
            cur.append(line)
    return names, ["".join(s) for s in seqs]


@dataclass
class Dataset:
    """Alignment and rooted binary tree (src/Dataset.jl:99-199)."""
    names: List[str]
    sequences: List[str]
    masks: np.ndarray            # uint8 [numseqs, numcols]
    gapfrequency: np.ndarray     # float64 [numcols]
    obsfreqs: np.ndarray         # float64 [4]
    children: np.ndarray         # int32 [numnodes, 2], -1 for leaves
    seqindex: np.ndarray         # int32 [numnodes], -1 for internal nodes
    branchlengths: np.ndarray    # float64 [numnodes], branch above each node
    parent: np.ndarray           # int32 [numnodes], -1 for the root
    root: Optional[TreeNode] = field(default=None, repr=False)

    @property
    def numseqs(self):
        return self.masks.shape[0]

    @property
    def numcols(self):
        return self.masks.shape[1]

    @property
    def numnodes(self):
        return self.children.shape[0]

    @classmethod
    def from_fasta_newick(cls, fasta_text: str, newick_text: str, doroottree=True):
        names, seqs = parse_fasta(fasta_text)
        return cls.from_sequences(names, seqs, newick_text.strip().splitlines()[0], doroottree)

    @classmethod
    def from_sequences(cls, names, seqs, newick: str, doroottree=True):
        if not seqs:
            raise ValueError("empty alignment")
        L = len(seqs[0])
        if any(len(s) != L for s in seqs):
            raise ValueError("sequences are not aligned (unequal lengths)")
        if all(s.isascii() for s in seqs):
            # byte lookup tables (same mapping as char_mask / NUCMAPPING)
            raw = np.frombuffer("".join(seqs).encode("ascii"), dtype=np.uint8).reshape(len(seqs), L)
            masks = _MASK_LUT[raw]
            nuc = _NUC_LUT[raw]
        else:
            masks = np.array([[char_mask(c) for c in s] for s in seqs], dtype=np.uint8).reshape(len(seqs), L)
            nuc = np.array([[NUCMAPPING.get(c, -1) for c in s] for s in seqs], dtype=np.int8).reshape(len(seqs), L)
        gap = (nuc < 0).astype(np.float64)
        obs = np.bincount(nuc[nuc >= 0].astype(np.int64), minlength=4).astype(np.float64)[:4]
        obs = obs / obs.sum() if obs.sum() > 0 else np.full(4, 0.25)
        root = parse_newick(newick)
        if doroottree:
            root = roottree(root, 0)
        nameidx = {n: i for i, n in enumerate(names)}
        nodes = getnodelist(root)
        for k, n in enumerate(nodes):
            n.nodeindex = k
            n.seqindex = nameidx.get(n.name, -1) if n.isleaf() else -1
        children = np.full((len(nodes), 2), -1, dtype=np.int32)
        parent = np.full(len(nodes), -1, dtype=np.int32)
        seqindex = np.full(len(nodes), -1, dtype=np.int32)
        bl = np.zeros(len(nodes))
        for n in nodes:
            if n.isleaf():
                if n.seqindex < 0:
                    raise ValueError(f"tree leaf {n.name!r} has no sequence")
                seqindex[n.nodeindex] = n.seqindex
            else:
                if len(n.children) != 2:
                    raise ValueError(f"node {n.nodeindex} has {len(n.children)} children; the likelihood "
                                     "needs a binary tree after rooting (give an unrooted, trifurcating Newick)")
                children[n.nodeindex] = [n.children[0].nodeindex, n.children[1].nodeindex]
            for c in n.children:
                parent[c.nodeindex] = n.nodeindex
            bl[n.nodeindex] = n.branchlength
        return cls(names=list(names), sequences=list(seqs), masks=masks, gapfrequency=gap.mean(axis=0),
                   obsfreqs=obs, children=children, seqindex=seqindex, branchlengths=bl, parent=parent, root=root)

    def tree_arrays(self):
        return dict(children=self.children, seqindex=self.seqindex, branchlengths=self.branchlengths)
