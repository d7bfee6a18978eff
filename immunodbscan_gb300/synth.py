"""Seeded synthetic immune repertoires for the five benchmark workloads.

No public dataset is involved: these generators stand in for the repertoires the
clustering path is measured on.  Every workload is a set of clonal families.  A
family has a root CDR3 and a V and J gene call; its members are copies of the
root with Poisson substitutions (and, for some workloads, single-residue or
single-codon indels).  Gene calls are IMGT-style strings
("Homsap IGHV3-23*01 F, or Homsap IGHV3-30*01 F") whose ambiguity sets hold 1-3
genes, so that the substring gene matching of the clustering path recovers
multi-bit V/J bitsets.

Workloads (``workload(k, scale=1.0, seed=...)``):
  0  10,000 aa CDR3s, 1,000 families of Geometric(0.1) size, Hamming eps=1, minPts=2
  1  200,000 nt CDR3s (24-75 nt, codon steps), 15,000 Zipf(1.5) families,
     Poisson(2) substitutions + 5% single-codon indels, Levenshtein eps=2, minPts=3
  2  64 aa repertoires, log-uniform sizes 5k-500k (~6M), per-repertoire clonality
     Zipf(U(1.2,2.0)), Hamming eps=1, minPts=2
  3  2,000,000 aa, V/J usage Zipf(1.8), Levenshtein eps=2, minPts=2
  4  10,000,000 aa, lengths Normal(16,3.5), 50,000 Zipf(1.3) families,
     Poisson(1.5) substitutions + 3% indels, eps = min(3, trunc(0.15*L)), minPts=4
``scale`` shrinks row counts (and family counts) proportionally for tests.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

AA = b"ACDEFGHIKLMNPQRSTVWY"
NT = b"ACGT"


@dataclasses.dataclass
class Workload:
    """Column-major rows plus the clustering parameters of one workload."""

    name: str
    seq_blob: np.ndarray          # uint8, concatenated sequences
    seq_off: np.ndarray           # int64 [n+1]
    v_blob: np.ndarray            # uint8, concatenated V calls
    v_off: np.ndarray             # int64 [n+1]
    j_blob: np.ndarray
    j_off: np.ndarray
    v_genes: List[bytes]
    j_genes: List[bytes]
    threshold: float              # NaN = relative threshold not used
    abs_eps: int                  # -1 = absolute eps not used
    min_pts: int
    use_hamming: bool
    rep_off: np.ndarray           # uint32 [R+1]
    alphabet: bytes = AA
    seed: int = 0
    candidates: int = 0           # 0 = automatic candidate pairs, 1 = buckets only
    edge_memory_mb: int = 0       # neighbour-pair list memory (0 no limit, < 0 streamed)
    row_chunks: int = 0           # host columns copied in this many row chunks (0 automatic)

    @property
    def n(self) -> int:
        return int(self.seq_off.shape[0] - 1)

    @property
    def n_rep(self) -> int:
        return int(self.rep_off.shape[0] - 1)

    def seq(self, i: int) -> bytes:
        return self.seq_blob[self.seq_off[i]:self.seq_off[i + 1]].tobytes()

    def vcall(self, i: int) -> bytes:
        return self.v_blob[self.v_off[i]:self.v_off[i + 1]].tobytes()

    def jcall(self, i: int) -> bytes:
        return self.j_blob[self.j_off[i]:self.j_off[i + 1]].tobytes()

    def lengths(self) -> np.ndarray:
        return np.diff(self.seq_off)

    def subset_repertoires(self, reps: Sequence[int]) -> "Workload":
        """A workload made of the given repertoires (row order kept)."""
        rows = [np.arange(self.rep_off[r], self.rep_off[r + 1]) for r in reps]
        sizes = [len(x) for x in rows]
        idx = np.concatenate(rows) if rows else np.zeros(0, np.int64)
        out = take_rows(self, idx)
        out.rep_off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
        return out


def _gather_strings(blob: np.ndarray, off: np.ndarray, idx: np.ndarray):
    """Concatenate strings idx[k] of (blob, off) into a new (blob, off)."""
    idx = np.asarray(idx, dtype=np.int64)
    starts = off[idx]
    lens = off[idx + 1] - starts
    new_off = np.zeros(len(idx) + 1, np.int64)
    np.cumsum(lens, out=new_off[1:])
    total = int(new_off[-1])
    if total == 0:
        return np.zeros(0, np.uint8), new_off
    # flat source index = start of the string + position within it
    seg = np.repeat(np.arange(len(idx)), lens)
    pos = np.arange(total, dtype=np.int64) - new_off[seg]
    return blob[starts[seg] + pos], new_off


def take_rows(w: Workload, idx: np.ndarray) -> Workload:
    """A one-repertoire workload holding rows idx of w (in the given order)."""
    sb, so = _gather_strings(w.seq_blob, w.seq_off, idx)
    vb, vo = _gather_strings(w.v_blob, w.v_off, idx)
    jb, jo = _gather_strings(w.j_blob, w.j_off, idx)
    return dataclasses.replace(w, seq_blob=sb, seq_off=so, v_blob=vb, v_off=vo,
                               j_blob=jb, j_off=jo,
                               rep_off=np.array([0, len(idx)], np.uint32))


def gene_names(prefix: str, n: int) -> List[bytes]:
    """n IMGT-like gene names ending in '*' ("IGHV3-23*"), none a prefix of another
    before the '*'."""
    names = []
    fam = 1
    num = 1
    while len(names) < n:
        if prefix.endswith("J"):
            names.append(f"{prefix}{len(names) + 1}*".encode())
            continue
        names.append(f"{prefix}{fam}-{num}*".encode())
        num += 1 + (num % 3 == 0)
        if num > 70:
            fam += 1
            num = 1
    return names


def _split_sizes(raw: np.ndarray, total: int) -> np.ndarray:
    """Rescale positive raw sizes to integers >= 1 summing to total."""
    raw = np.asarray(raw, dtype=np.float64)
    k = len(raw)
    if k > total:
        raw = raw[:total]
        k = total
    base = np.ones(k, np.int64)
    rest = total - k
    if rest > 0:
        share = raw / raw.sum() * rest
        fl = np.floor(share).astype(np.int64)
        rem = rest - int(fl.sum())
        order = np.argsort(-(share - fl), kind="stable")
        fl[order[:rem]] += 1
        base += fl
    return base


def _pick_sets(rng, n_sets: int, n_genes: int, usage: Optional[np.ndarray]) -> np.ndarray:
    """n_sets gene sets of 1-3 distinct genes (weighted by `usage` if given), as
    bitmasks (uint64 words, one row per set).  Sampling without replacement by
    the Gumbel top-k rule."""
    k = rng.integers(1, 4, size=n_sets)
    logp = np.log(usage) if usage is not None else np.zeros(n_genes)
    keys = logp[None, :] + rng.gumbel(size=(n_sets, n_genes))
    top = np.argsort(-keys, axis=1)[:, :3]
    nw = (n_genes + 63) // 64
    masks = np.zeros((n_sets, nw), np.uint64)
    for slot in range(min(3, n_genes)):
        sel = k > slot
        g = top[sel, slot]
        np.bitwise_or.at(masks, (np.nonzero(sel)[0], g // 64), np.uint64(1) << (g % 64).astype(np.uint64))
    return masks


def _call_strings(rng, masks: np.ndarray, names: List[bytes], species=b"Homsap ") -> List[bytes]:
    """IMGT-style call string for each gene bitmask, alleles *01-*03 drawn at random."""
    tokens = [[species + names[g] + b"%02d F" % a for a in (1, 2, 3)] for g in range(len(names))]
    alle = rng.integers(0, 3, size=(len(masks), 4))
    out = []
    for i in range(len(masks)):
        parts = []
        t = 0
        for w in range(masks.shape[1]):
            m = int(masks[i, w])
            while m:
                low = m & -m
                g = w * 64 + low.bit_length() - 1
                parts.append(tokens[g][alle[i, t & 3]])
                t += 1
                m ^= low
        out.append(b", or ".join(parts))
    return out


def _zipf_usage(n: int, a: float) -> np.ndarray:
    w = 1.0 / np.arange(1, n + 1, dtype=np.float64) ** a
    return w / w.sum()


def _families(rng, *, n_rows: int, n_fam: int, sizes: str, size_param: float,
              len_mu: float, len_sd: float, len_lo: int, len_hi: int,
              alphabet: bytes, codon: bool, sub_rate: float, indel_rate: float,
              v_names: List[bytes], j_names: List[bytes],
              v_usage: Optional[np.ndarray], j_usage: Optional[np.ndarray],
              variant_rate: float = 0.1):
    """One repertoire of n_rows rows drawn from n_fam clonal families."""
    A = len(alphabet)
    alpha = np.frombuffer(alphabet, dtype=np.uint8)
    if sizes == "geometric":
        raw = rng.geometric(size_param, size=n_fam)
    else:
        raw = np.minimum(rng.zipf(size_param, size=n_fam), 10 * n_rows).astype(np.float64)
    fam_size = _split_sizes(raw, n_rows)
    n_fam = len(fam_size)
    # root lengths
    if codon:
        L = rng.integers(len_lo // 3, len_hi // 3 + 1, size=n_fam) * 3
    else:
        L = np.clip(np.rint(rng.normal(len_mu, len_sd, size=n_fam)), len_lo, len_hi).astype(np.int64)
    Lmax = int(len_hi) + (3 if codon else 1)
    # position x residue frequency table (fixed per repertoire seed)
    if codon:
        freq = np.full((Lmax, A), 1.0 / A)
    else:
        freq = rng.dirichlet(np.full(A, 0.6), size=Lmax)
    cdf = np.cumsum(freq, axis=1)
    cdf[:, -1] = 1.0

    def draw(pos: np.ndarray) -> np.ndarray:
        u = rng.random(len(pos))
        c = cdf[pos]
        return (u[:, None] > c).sum(axis=1).clip(0, A - 1).astype(np.uint8)

    roots = np.zeros((n_fam, Lmax), np.uint8)
    pos_grid = np.broadcast_to(np.arange(Lmax), (n_fam, Lmax))
    roots[:] = draw(pos_grid.reshape(-1)).reshape(n_fam, Lmax)
    # members
    fam = np.repeat(np.arange(n_fam), fam_size)
    rng.shuffle(fam)
    n = len(fam)
    seqs = roots[fam].copy()
    lens = L[fam].copy()
    k = rng.poisson(sub_rate, size=n)
    rows = np.repeat(np.arange(n), k)
    p = (rng.random(len(rows)) * lens[rows]).astype(np.int64)
    seqs[rows, p] = draw(p)
    # indels (single residue, or single codon for nucleotides)
    step = 3 if codon else 1
    ind = np.nonzero(rng.random(n) < indel_rate)[0]
    for i in ind:
        li = int(lens[i])
        s = seqs[i, :li].tolist()
        if rng.random() < 0.5 and li - step >= max(step, 1):
            q = int(rng.integers(0, li // step)) * step
            del s[q:q + step]
        elif li + step <= Lmax:
            q = int(rng.integers(0, li // step + 1)) * step
            s[q:q] = [int(x) for x in rng.integers(0, A, size=step)]
        seqs[i, :] = 0
        seqs[i, :len(s)] = s
        lens[i] = len(s)
    # encode sequences
    mask = np.arange(Lmax)[None, :] < lens[:, None]
    seq_blob = alpha[seqs[mask]].astype(np.uint8)
    seq_off = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=seq_off[1:])
    # gene calls: every family has a main call and a variant call (one gene more)
    vsets = _pick_sets(rng, n_fam, len(v_names), v_usage)
    jsets = _pick_sets(rng, n_fam, len(j_names), j_usage)

    def variants(masks, n_genes):
        # the family's set plus one random gene (possibly already in it)
        extra = rng.integers(0, n_genes, size=len(masks))
        out = masks.copy()
        np.bitwise_or.at(out, (np.arange(len(masks)), extra // 64),
                         np.uint64(1) << (extra % 64).astype(np.uint64))
        return out

    vcall = _call_strings(rng, np.concatenate([vsets, variants(vsets, len(v_names))]), v_names)
    jcall = _call_strings(rng, np.concatenate([jsets, variants(jsets, len(j_names))]), j_names)
    which_v = fam + n_fam * (rng.random(n) < variant_rate)
    which_j = fam + n_fam * (rng.random(n) < variant_rate)

    def blobify(strs, which):
        lens_ = np.array([len(s) for s in strs], np.int64)
        off_ = np.zeros(len(strs) + 1, np.int64)
        np.cumsum(lens_, out=off_[1:])
        blob_ = np.frombuffer(b"".join(strs), dtype=np.uint8)
        return _gather_strings(blob_, off_, which)

    vb, vo = blobify(vcall, which_v)
    jb, jo = blobify(jcall, which_j)
    return seq_blob, seq_off, vb, vo, jb, jo


def _concat(parts):
    blobs, offs = [], []
    base = 0
    for b, o in parts:
        blobs.append(b)
        offs.append(o[:-1] + base)
        base += int(o[-1])
    off = np.concatenate(offs + [np.array([base], np.int64)])
    return np.concatenate(blobs) if blobs else np.zeros(0, np.uint8), off


def workload(k: int, scale: float = 1.0, seed: Optional[int] = None) -> Workload:
    """Synthetic workload k (0..4) at the given scale (1.0 = full size)."""
    seed = 1000 + k if seed is None else seed
    rng = np.random.default_rng(seed)
    nan = float("nan")
    if k == 0:
        vn, jn = gene_names("IGHV", 50), gene_names("IGHJ", 6)
        n = max(int(10_000 * scale), 2)
        parts = [_families(rng, n_rows=n, n_fam=max(int(1000 * scale), 1), sizes="geometric",
                           size_param=0.1, len_mu=15, len_sd=3, len_lo=8, len_hi=25,
                           alphabet=AA, codon=False, sub_rate=1.0, indel_rate=0.0,
                           v_names=vn, j_names=jn, v_usage=None, j_usage=None)]
        prm = dict(threshold=nan, abs_eps=1, min_pts=2, use_hamming=True, alphabet=AA)
    elif k == 1:
        vn, jn = gene_names("IGHV", 60), gene_names("IGHJ", 6)
        n = max(int(200_000 * scale), 2)
        parts = [_families(rng, n_rows=n, n_fam=max(int(15_000 * scale), 1), sizes="zipf",
                           size_param=1.5, len_mu=0, len_sd=0, len_lo=24, len_hi=75,
                           alphabet=NT, codon=True, sub_rate=2.0, indel_rate=0.05,
                           v_names=vn, j_names=jn, v_usage=None, j_usage=None)]
        prm = dict(threshold=nan, abs_eps=2, min_pts=3, use_hamming=False, alphabet=NT)
    elif k == 2:
        vn, jn = gene_names("IGHV", 50), gene_names("IGHJ", 6)
        R = 64
        sizes = np.exp(rng.uniform(math.log(5_000), math.log(500_000), size=R))
        sizes = np.maximum((sizes * scale).astype(np.int64), 2)
        parts = []
        for r in range(R):
            a = float(rng.uniform(1.2, 2.0))
            nr = int(sizes[r])
            parts.append(_families(rng, n_rows=nr, n_fam=max(nr // 10, 1), sizes="zipf",
                                   size_param=a, len_mu=15, len_sd=3, len_lo=8, len_hi=25,
                                   alphabet=AA, codon=False, sub_rate=1.0, indel_rate=0.0,
                                   v_names=vn, j_names=jn, v_usage=None, j_usage=None))
        prm = dict(threshold=nan, abs_eps=1, min_pts=2, use_hamming=True, alphabet=AA)
    elif k == 3:
        vn, jn = gene_names("IGHV", 50), gene_names("IGHJ", 6)
        n = max(int(2_000_000 * scale), 2)
        parts = [_families(rng, n_rows=n, n_fam=max(int(200_000 * scale), 1), sizes="zipf",
                           size_param=1.8, len_mu=15, len_sd=3, len_lo=8, len_hi=25,
                           alphabet=AA, codon=False, sub_rate=1.0, indel_rate=0.02,
                           v_names=vn, j_names=jn, v_usage=_zipf_usage(50, 1.8),
                           j_usage=_zipf_usage(6, 1.8))]
        prm = dict(threshold=nan, abs_eps=2, min_pts=2, use_hamming=False, alphabet=AA)
    elif k == 4:
        vn, jn = gene_names("IGHV", 50), gene_names("IGHJ", 6)
        n = max(int(10_000_000 * scale), 2)
        parts = [_families(rng, n_rows=n, n_fam=max(int(50_000 * scale), 1), sizes="zipf",
                           size_param=1.3, len_mu=16, len_sd=3.5, len_lo=4, len_hi=36,
                           alphabet=AA, codon=False, sub_rate=1.5, indel_rate=0.03,
                           v_names=vn, j_names=jn, v_usage=None, j_usage=None)]
        prm = dict(threshold=0.15, abs_eps=3, min_pts=4, use_hamming=False, alphabet=AA)
    else:
        raise ValueError(f"unknown workload {k}")
    sb, so = _concat([(p[0], p[1]) for p in parts])
    vb, vo = _concat([(p[2], p[3]) for p in parts])
    jb, jo = _concat([(p[4], p[5]) for p in parts])
    rep_sizes = [len(p[1]) - 1 for p in parts]
    rep_off = np.concatenate([[0], np.cumsum(rep_sizes)]).astype(np.uint32)
    return Workload(name=f"workload{k}", seq_blob=sb, seq_off=so, v_blob=vb, v_off=vo,
                    j_blob=jb, j_off=jo, v_genes=vn, j_genes=jn, rep_off=rep_off,
                    seed=seed, **prm)


def from_strings(seqs: Sequence[bytes], vcalls: Optional[Sequence[bytes]],
                 jcalls: Optional[Sequence[bytes]], v_genes: Sequence[bytes],
                 j_genes: Sequence[bytes], *, threshold=float("nan"), abs_eps=-1,
                 min_pts=2, use_hamming=False, rep_sizes=None) -> Workload:
    """Build a workload from Python byte strings (small hand-written cases)."""
    def blob(strs):
        strs = list(strs)
        off = np.zeros(len(strs) + 1, np.int64)
        np.cumsum([len(s) for s in strs], out=off[1:])
        return np.frombuffer(b"".join(strs), dtype=np.uint8).copy(), off

    sb, so = blob(seqs)
    n = len(seqs)
    vb, vo = blob(vcalls if vcalls is not None else [b"V"] * n)
    jb, jo = blob(jcalls if jcalls is not None else [b"V"] * n)
    if rep_sizes is None:
        rep_sizes = [n]
    rep_off = np.concatenate([[0], np.cumsum(rep_sizes)]).astype(np.uint32)
    return Workload(name="custom", seq_blob=sb, seq_off=so, v_blob=vb, v_off=vo,
                    j_blob=jb, j_off=jo,
                    v_genes=list(v_genes) if vcalls is not None else [b"V"],
                    j_genes=list(j_genes) if jcalls is not None else [b"V"],
                    threshold=threshold, abs_eps=abs_eps, min_pts=min_pts,
                    use_hamming=use_hamming, rep_off=rep_off)
