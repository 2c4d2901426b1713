"""Par-CD binary graph format ("PCD") and the seeded synthetic workloads.

File layout written by the reference converter (src/convert.cpp:244-278) and
read by src/graph.cpp:40-105, all little-endian int32 with no padding:

    "PCD"                3 bytes of magic
    n, m                 vertices, undirected edges
    indices[n + 1]       CSR row offsets (indices[n] == 2m)
    adj[2m]              neighbours, each row sorted ascending, no loops/duplicates
    map[n]               original vertex id of each new id

`convert_edges` restates the converter's pipeline (src/convert.cpp:76-196):
text edges -> symmetric CSR -> per-row sort + duplicate/loop removal ->
relabel by (degree, id) descending -> rows re-sorted -> trailing isolated
vertices dropped.  The one deliberate difference is that self-loops are removed
before the CSR is built: the reference's `convert_to_csr` writes a loop's slot
twice and leaves another uninitialised (src/convert.cpp:97-102), so inputs with
loops are not valid inputs for it.  On loop-free input the bytes written here
are identical to the reference converter's (checked by the tests).

Generators (all seeded, loop/duplicate free):
  * `sbm`       planted partition / stochastic block model
  * `rmat`      R-MAT with quadrant probabilities (a, b, c, d) and a random
                vertex permutation
  * `powerlaw`  LFR-style planted communities: power-law degrees and
                community sizes, mixing parameter mu
  * `sbm_batch` the log-normal-size batch of SBMs
Each returns an (E, 2) int64 array of undirected edges (a < b not required).
"""
from __future__ import annotations

import io
import struct
from dataclasses import dataclass

import numpy as np

MAGIC = b"PCD"


@dataclass
class CSRGraph:
    """Undirected graph in the reference's CSR layout (src/graph.hpp:6-40)."""

    n: int
    m: int
    indices: np.ndarray  # int32[n + 1]
    adj: np.ndarray      # int32[2m]
    map: np.ndarray      # int32[n]

    def degree(self) -> np.ndarray:
        return np.diff(self.indices).astype(np.int32)


# --------------------------------------------------------------------------
# PCD file I/O
# --------------------------------------------------------------------------

def to_bytes(g: CSRGraph) -> bytes:
    """Serialise exactly as src/convert.cpp:244-256 writes the file."""
    buf = io.BytesIO()
    buf.write(MAGIC)
    buf.write(struct.pack("<ii", g.n, g.m))
    buf.write(np.ascontiguousarray(g.indices, dtype="<i4").tobytes())
    buf.write(np.ascontiguousarray(g.adj, dtype="<i4").tobytes())
    buf.write(np.ascontiguousarray(g.map, dtype="<i4").tobytes())
    return buf.getvalue()


def write_pcd(path: str, g: CSRGraph) -> None:
    with open(path, "wb") as f:
        f.write(to_bytes(g))


class FormatError(ValueError):
    """The file is not a well-formed PCD graph (mirrors Graph::read returning NULL)."""


def from_bytes(data: bytes) -> CSRGraph:
    """Parse a PCD file with the checks of src/graph.cpp:40-105: magic, header,
    exact length (no trailing bytes), plus the structural checks the reference
    leaves implicit (monotone offsets, neighbour ids in range)."""
    if len(data) < 11 or data[:3] != MAGIC:
        raise FormatError("invalid file type")
    n, m = struct.unpack_from("<ii", data, 3)
    if n < 0 or m < 0:
        raise FormatError("negative header")
    need = 11 + 4 * (n + 1) + 8 * m + 4 * n
    if len(data) != need:
        raise FormatError(f"file length {len(data)} != expected {need}")
    off = 11
    indices = np.frombuffer(data, dtype="<i4", count=n + 1, offset=off).astype(np.int32)
    off += 4 * (n + 1)
    adj = np.frombuffer(data, dtype="<i4", count=2 * m, offset=off).astype(np.int32)
    off += 8 * m
    mp = np.frombuffer(data, dtype="<i4", count=n, offset=off).astype(np.int32)
    g = CSRGraph(n, m, indices, adj, mp)
    validate(g)
    return g


def read_pcd(path: str) -> CSRGraph:
    with open(path, "rb") as f:
        return from_bytes(f.read())


def validate(g: CSRGraph) -> None:
    if g.indices.shape[0] != g.n + 1 or g.adj.shape[0] != 2 * g.m:
        raise FormatError("array sizes do not match header")
    if g.n and (g.indices[0] != 0 or g.indices[-1] != 2 * g.m):
        raise FormatError("row offsets do not span the adjacency")
    if g.n and np.any(np.diff(g.indices.astype(np.int64)) < 0):
        raise FormatError("row offsets are not monotone")
    if g.m and (g.adj.min() < 0 or g.adj.max() >= g.n):
        raise FormatError("neighbour id out of range")


# --------------------------------------------------------------------------
# the converter pipeline
# --------------------------------------------------------------------------

def convert_edges(edges: np.ndarray, num_nodes: int | None = None) -> CSRGraph:
    """Edge list -> CSRGraph with the reference converter's semantics.

    num_nodes defaults to max id + 1 (src/convert.cpp:61).
    """
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    if num_nodes is None:
        num_nodes = int(e.max()) + 1 if e.size else 0
    a, b = e[:, 0], e[:, 1]
    keep = a != b
    a, b = a[keep], b[keep]
    # symmetric, deduplicated (row, col) pairs  (convert.cpp:76-133)
    rows = np.concatenate([a, b])
    cols = np.concatenate([b, a])
    key = np.unique(rows * num_nodes + cols)
    rows = key // num_nodes
    cols = key % num_nodes
    deg = np.bincount(rows, minlength=num_nodes).astype(np.int64)
    # relabel by (degree, id) descending  (convert.cpp:136-156)
    order = np.lexsort((-np.arange(num_nodes), -deg))
    new_id = np.empty(num_nodes, dtype=np.int64)
    new_id[order] = np.arange(num_nodes)
    r2 = new_id[rows]
    c2 = new_id[cols]
    key2 = np.sort(r2 * num_nodes + c2)
    r2 = key2 // num_nodes
    c2 = key2 % num_nodes
    deg2 = deg[order]
    # drop trailing isolated vertices  (convert.cpp:184-196)
    nz = np.nonzero(deg2 == 0)[0]
    n = int(nz[0]) if nz.size else num_nodes
    indices = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg2[:n], out=indices[1:])
    m = int(indices[-1] // 2)
    return CSRGraph(
        n=n,
        m=m,
        indices=indices.astype(np.int32),
        adj=c2.astype(np.int32),
        map=order[:n].astype(np.int32),
    )


def edges_to_text(edges: np.ndarray) -> str:
    e = np.asarray(edges, dtype=np.int64).reshape(-1, 2)
    return "".join(f"{int(x)} {int(y)}\n" for x, y in e)


def from_csr(indices, adj) -> CSRGraph:
    """Wrap an already-valid CSR (identity map)."""
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    adj = np.ascontiguousarray(adj, dtype=np.int32)
    n = indices.shape[0] - 1
    g = CSRGraph(n, adj.shape[0] // 2, indices, adj, np.arange(n, dtype=np.int32))
    validate(g)
    return g


# --------------------------------------------------------------------------
# generators
# --------------------------------------------------------------------------

def _dedup_undirected(a: np.ndarray, b: np.ndarray, n: int) -> np.ndarray:
    keep = a != b
    a, b = a[keep], b[keep]
    lo = np.minimum(a, b)
    hi = np.maximum(a, b)
    key = np.unique(lo * n + hi)
    return np.stack([key // n, key % n], axis=1)


def sbm(n_blocks: int, block_size: int, p_in: float, p_out: float, seed: int) -> np.ndarray:
    """Planted partition with equal blocks; every pair is an independent
    Bernoulli trial (p_in inside a block, p_out across).  Exact per-pair
    sampling, so only for modest n (the 10k-vertex workload)."""
    rng = np.random.default_rng(seed)
    n = n_blocks * block_size
    out = []
    blk = np.arange(n) // block_size
    chunk = max(1, 4_000_000 // n)
    for i0 in range(0, n, chunk):
        i1 = min(n, i0 + chunk)
        ii = np.arange(i0, i1)[:, None]
        jj = np.arange(n)[None, :]
        p = np.where(blk[ii] == blk[jj], p_in, p_out)
        hit = (rng.random((i1 - i0, n)) < p) & (jj > ii)
        a, b = np.nonzero(hit)
        out.append(np.stack([a + i0, b], axis=1))
    return np.concatenate(out).astype(np.int64)


def sbm_sparse(sizes: np.ndarray, deg_in: float, deg_out: float, rng) -> np.ndarray:
    """SBM by edge counts: block s gets Binomial(s(s-1)/2, p_in) distinct
    intra pairs with p_in = deg_in/(s-1); inter pairs are drawn uniformly over
    pairs in different blocks with expected mean inter-degree deg_out."""
    sizes = np.asarray(sizes, dtype=np.int64)
    n = int(sizes.sum())
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    a_parts, b_parts = [], []
    for s, st in zip(sizes, starts):
        if s < 2:
            continue
        pairs = s * (s - 1) // 2
        p = min(1.0, deg_in / (s - 1))
        k = rng.binomial(pairs, p)
        if k == 0:
            continue
        u = st + rng.integers(0, s, size=int(k * 1.1) + 4)
        v = st + rng.integers(0, s, size=u.shape[0])
        a_parts.append(u)
        b_parts.append(v)
    k_out = rng.poisson(deg_out * n / 2.0)
    if k_out and len(sizes) > 1:
        blk = np.repeat(np.arange(len(sizes)), sizes)
        u = rng.integers(0, n, size=k_out)
        v = rng.integers(0, n, size=k_out)
        ok = blk[u] != blk[v]
        a_parts.append(u[ok])
        b_parts.append(v[ok])
    if not a_parts:
        return np.zeros((0, 2), dtype=np.int64)
    return _dedup_undirected(np.concatenate(a_parts), np.concatenate(b_parts), n)


def rmat(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int) -> np.ndarray:
    """R-MAT edges (numpy; for test-sized scales).  Vertex ids are randomly
    permuted; loops and duplicates removed."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    ne = edge_factor * n
    src = np.zeros(ne, dtype=np.int64)
    dst = np.zeros(ne, dtype=np.int64)
    ab, abc = a + b, a + b + c
    for lvl in range(scale):
        r = rng.random(ne)
        bit_s = (r >= ab).astype(np.int64)
        bit_d = (((r >= a) & (r < ab)) | (r >= abc)).astype(np.int64)
        src |= bit_s << lvl
        dst |= bit_d << lvl
    perm = rng.permutation(n)
    return _dedup_undirected(perm[src], perm[dst], n)


def rmat_torch(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int,
               device="cuda"):
    """R-MAT generated on a device with torch (input generation for the large
    benchmark workloads only).  Returns (indices, adj, map) as numpy int32 with
    the converter's semantics (degree-sorted, isolated vertices dropped)."""
    src, dst = rmat_edges_torch(scale, edge_factor, a, b, c, seed, device)
    return csr_from_edges_torch(src, dst, 1 << scale)


def rmat_edges_torch(scale: int, edge_factor: int, a: float, b: float, c: float, seed: int, device="cuda"):
    """The raw R-MAT edge list of rmat_torch (with loops and duplicates), as
    two int64 device tensors."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    n = 1 << scale
    ne = edge_factor * n
    src = torch.zeros(ne, dtype=torch.int64, device=device)
    dst = torch.zeros(ne, dtype=torch.int64, device=device)
    ab, abc = a + b, a + b + c
    chunk = 1 << 26
    for lvl in range(scale):
        for s0 in range(0, ne, chunk):
            s1 = min(ne, s0 + chunk)
            r = torch.rand(s1 - s0, generator=gen, device=device)
            bs = (r >= ab).to(torch.int64)
            bd = (((r >= a) & (r < ab)) | (r >= abc)).to(torch.int64)
            src[s0:s1] |= bs << lvl
            dst[s0:s1] |= bd << lvl
            del r, bs, bd
    perm = torch.randperm(n, generator=gen, device=device)
    src = perm[src]
    dst = perm[dst]
    del perm
    return src, dst


def csr_from_edges_torch(src, dst, n):
    """Converter semantics on the device (torch): loops dropped, symmetric,
    deduplicated, relabelled by (degree, id) descending, rows sorted, trailing
    isolated vertices removed.  Returns numpy (indices, adj, map)."""
    import torch

    keep = src != dst
    src, dst = src[keep], dst[keep]
    lo = torch.minimum(src, dst)
    hi = torch.maximum(src, dst)
    del src, dst, keep
    key = torch.unique(lo * n + hi)
    del lo, hi
    lo = key // n
    hi = key % n
    del key
    deg = torch.bincount(lo, minlength=n) + torch.bincount(hi, minlength=n)
    ids = torch.arange(n, device=deg.device)
    # sort by (deg desc, id desc): key = deg * n + id, descending
    order = torch.argsort(deg * n + ids, descending=True)
    new_id = torch.empty_like(order)
    new_id[order] = ids
    lo = new_id[lo]
    hi = new_id[hi]
    rows = torch.cat([lo, hi])
    cols = torch.cat([hi, lo])
    del lo, hi
    key = torch.sort(rows * n + cols).values
    del rows
    cols = (key % n).to(torch.int32)
    rows_sorted = key // n
    del key
    deg2 = deg[order]
    nz = torch.nonzero(deg2 == 0)
    nn = int(nz[0, 0]) if nz.numel() else n
    counts = torch.bincount(rows_sorted, minlength=n)[:nn]
    del rows_sorted
    indices = torch.zeros(nn + 1, dtype=torch.int64, device=deg.device)
    indices[1:] = torch.cumsum(counts, 0)
    out = (indices.to(torch.int32).cpu().numpy(), cols.cpu().numpy(),
           order[:nn].to(torch.int32).cpu().numpy())
    return out


def powerlaw_sample(rng, n, exponent, lo, hi):
    """Inverse-CDF sampling of a continuous power law x^-exponent on [lo, hi],
    rounded down to integers."""
    u = rng.random(n)
    e1 = 1.0 - exponent
    x = (lo ** e1 + u * (hi ** e1 - lo ** e1)) ** (1.0 / e1)
    return np.floor(x).astype(np.int64)


def powerlaw(n: int, deg_exp: float, deg_min: int, deg_max: int, comm_exp: float,
             comm_min: int, comm_max: int, mu: float, seed: int) -> np.ndarray:
    """LFR-style planted communities (our own construction, not networkx's
    LFR): degrees and community sizes are power laws; each vertex sends a
    fraction (1 - mu) of its stubs inside its community and mu outside; stubs
    are paired uniformly at random (configuration model) inside each community
    and globally for the outside stubs; loops and duplicates are dropped."""
    rng = np.random.default_rng(seed)
    deg = powerlaw_sample(rng, n, deg_exp, deg_min, deg_max)
    sizes = []
    tot = 0
    while tot < n:
        s = int(powerlaw_sample(rng, 1, comm_exp, comm_min, comm_max)[0])
        s = min(s, n - tot)
        sizes.append(s)
        tot += s
    sizes = np.array(sizes, dtype=np.int64)
    comm = np.repeat(np.arange(sizes.shape[0]), sizes)
    rng.shuffle(comm)
    k_in = np.rint(deg * (1.0 - mu)).astype(np.int64)
    k_out = deg - k_in
    # intra stubs: pair within community by sorting stubs on (community, random)
    stub_v = np.repeat(np.arange(n), k_in)
    stub_c = comm[stub_v]
    order = np.lexsort((rng.random(stub_v.shape[0]), stub_c))
    stub_v = stub_v[order]
    stub_c = stub_c[order]
    # pair consecutive stubs that share a community
    same = stub_c[:-1:2] == stub_c[1::2] if stub_v.shape[0] >= 2 else np.zeros(0, bool)
    a_in = stub_v[:-1:2][same]
    b_in = stub_v[1::2][same]
    # inter stubs: global random pairing, drop same-community pairs
    so = np.repeat(np.arange(n), k_out)
    rng.shuffle(so)
    h = so.shape[0] // 2
    a_out, b_out = so[:h], so[h:2 * h]
    ok = comm[a_out] != comm[b_out]
    a = np.concatenate([a_in, a_out[ok]])
    b = np.concatenate([b_in, b_out[ok]])
    return _dedup_undirected(a, b, n)


def powerlaw_torch(n: int, deg_exp: float, deg_min: int, deg_max: int, comm_exp: float, comm_min: int,
                   comm_max: int, mu: float, seed: int, device="cuda"):
    """The construction of `powerlaw` (LFR-style planted communities) with
    torch on a device, for the large power-law workloads (8 M vertices):
    power-law degrees and community sizes by inverse-CDF sampling, a fraction
    1 - mu of each vertex's stubs paired inside its community (stubs sorted
    by (community, random key), consecutive stubs of one community paired),
    the rest paired uniformly at random across the graph and kept when the two
    ends lie in different communities.  torch's random streams, so the graph
    differs from `powerlaw`'s draw for draw.  Returns numpy (indices, adj,
    map, community of each original vertex) with the converter's semantics."""
    import torch

    dev = torch.device(device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)

    def plaw(count, exponent, lo, hi):
        u = torch.rand(count, generator=gen, device=dev, dtype=torch.float64)
        e1 = 1.0 - exponent
        return torch.floor((lo ** e1 + u * (hi ** e1 - lo ** e1)) ** (1.0 / e1)).to(torch.int64)

    deg = plaw(n, deg_exp, deg_min, deg_max)
    # community sizes: draw until they cover n, the last one cut to fit
    sizes = plaw(2 * n // max(1, comm_min) + 16, comm_exp, comm_min, comm_max)
    cum = torch.cumsum(sizes, 0)
    ncomm = int(torch.searchsorted(cum, torch.tensor([n], device=dev, dtype=torch.int64)).item()) + 1
    sizes = sizes[:ncomm].clone()
    sizes[-1] -= int(cum[ncomm - 1].item()) - n
    comm = torch.repeat_interleave(torch.arange(ncomm, device=dev), sizes)
    comm = comm[torch.randperm(n, generator=gen, device=dev)]
    k_in = torch.round(deg.to(torch.float64) * (1.0 - mu)).to(torch.int64)
    k_out = deg - k_in
    ids = torch.arange(n, device=dev)
    # intra-community stubs
    sv = torch.repeat_interleave(ids, k_in)
    key = comm[sv] * (1 << 31) + torch.randint(0, 1 << 31, (sv.shape[0],), generator=gen, device=dev)
    sv = sv[torch.argsort(key)]
    del key
    h = sv.shape[0] // 2
    a_in, b_in = sv[0:2 * h:2], sv[1:2 * h:2]
    ok = comm[a_in] == comm[b_in]
    a_in, b_in = a_in[ok], b_in[ok]
    del sv, ok
    # inter-community stubs
    so = torch.repeat_interleave(ids, k_out)
    so = so[torch.randperm(so.shape[0], generator=gen, device=dev)]
    h = so.shape[0] // 2
    a_out, b_out = so[:h], so[h:2 * h]
    ok = comm[a_out] != comm[b_out]
    src = torch.cat([a_in, a_out[ok]])
    dst = torch.cat([b_in, b_out[ok]])
    del so, a_out, b_out, ok, a_in, b_in
    ind, adj, mp = csr_from_edges_torch(src, dst, n)
    return ind, adj, mp, comm.cpu().numpy()


def batch_sizes(count: int, median: float, sigma: float, lo: int, hi: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    s = np.exp(np.log(median) + sigma * rng.standard_normal(count))
    return np.clip(np.rint(s), lo, hi).astype(np.int64)


def sbm_batch(count: int = 4096, seed: int = 4, median: float = 5000, sigma: float = 1.2,
              lo: int = 200, hi: int = 300_000, deg_in: float = 12.0, deg_out: float = 2.0,
              block: int = 50):
    """The batched workload: `count` SBM graphs, log-normal vertex counts,
    n/block communities each, mean intra-degree deg_in, inter-degree deg_out.
    Yields CSRGraph objects (converter semantics) in order."""
    ns = batch_sizes(count, median, sigma, lo, hi, seed)
    rng = np.random.default_rng(seed + 1)
    for n in ns:
        nb = max(1, int(n) // block)
        sizes = np.full(nb, int(n) // nb, dtype=np.int64)
        sizes[: int(n) - int(sizes.sum())] += 1
        e = sbm_sparse(sizes, deg_in, deg_out, rng)
        yield convert_edges(e, int(n))


def sbm_batch_torch(count: int = 4096, seed: int = 4, median: float = 5000, sigma: float = 1.2,
                    lo: int = 200, hi: int = 300_000, deg_in: float = 12.0, deg_out: float = 2.0,
                    block: int = 50, device="cuda", sizes=None):
    """The batched SBM workload generated with torch on a device (input
    generation for the benchmark; `sbm_batch` is the numpy version for tests).

    Same laws as `sbm_batch`: log-normal vertex counts (`batch_sizes`), n/block
    near-equal blocks per graph, Binomial(s(s-1)/2, deg_in/(s-1)) intra pairs per
    block drawn with 10% oversampling, Poisson(deg_out*n/2) uniform inter pairs
    that are kept when their endpoints sit in different blocks.  The random
    streams are torch's, so the graphs differ from `sbm_batch`'s draw for draw.
    Every graph then gets the converter's semantics: loops and duplicates
    dropped, vertices relabelled by (degree, id) descending, isolated vertices
    removed.

    `sizes` (optional) gives the vertex counts directly instead of the
    log-normal law.

    Returns (vertex_offsets numpy int32[G+1], indices torch int32[N+1] union row
    offsets, adj torch int32[2M] local neighbour ids): the packed layout of
    pcd_batch_load_device."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    ns = batch_sizes(count, median, sigma, lo, hi, seed) if sizes is None else np.asarray(sizes, np.int64)
    G = ns.shape[0]
    nb = np.maximum(1, ns // block)
    base_sz = ns // nb
    extra = ns - base_sz * nb
    first_blk = np.cumsum(nb) - nb
    blk_local = np.arange(int(nb.sum())) - np.repeat(first_blk, nb)
    sz_np = np.repeat(base_sz, nb) + (blk_local < np.repeat(extra, nb))
    goff_np = np.concatenate([[0], np.cumsum(ns)]).astype(np.int64)
    N = int(goff_np[-1])
    dev = torch.device(device)
    sz = torch.from_numpy(sz_np.astype(np.int64)).to(dev)
    bstart = torch.cumsum(sz, 0) - sz            # graphs are contiguous, blocks tile them
    ns_t = torch.from_numpy(ns).to(dev)
    goff = torch.from_numpy(goff_np).to(dev)
    nblk = sz.shape[0]
    # intra-block pairs
    szf = sz.to(torch.float64)
    pairs = szf * (szf - 1) / 2
    p = torch.where(sz >= 2, torch.clamp(deg_in / torch.clamp(szf - 1, min=1.0), max=1.0), torch.zeros_like(szf))
    k = torch.binomial(pairs, p, generator=gen)
    draws = torch.where(sz >= 2, torch.floor(k * 1.1).to(torch.int64) + 4, torch.zeros_like(sz))
    rep = torch.repeat_interleave(torch.arange(nblk, device=dev), draws)
    s_rep = sz[rep]
    b_rep = bstart[rep]
    del rep

    def pick(size):
        r = torch.rand(size.shape[0], generator=gen, device=dev, dtype=torch.float64)
        return torch.minimum((r * size.to(torch.float64)).to(torch.int64), size - 1)

    a_in = b_rep + pick(s_rep)
    b_in = b_rep + pick(s_rep)
    del s_rep, b_rep
    # inter-block pairs
    k_out = torch.poisson(ns_t.to(torch.float64) * (deg_out / 2.0), generator=gen).to(torch.int64)
    grep = torch.repeat_interleave(torch.arange(G, device=dev), k_out)
    n_rep = ns_t[grep]
    g_rep = goff[grep]
    del grep
    a_out = g_rep + pick(n_rep)
    b_out = g_rep + pick(n_rep)
    del n_rep, g_rep
    vblk = torch.repeat_interleave(torch.arange(nblk, device=dev), sz)
    ok = vblk[a_out] != vblk[b_out]
    a = torch.cat([a_in, a_out[ok]])
    b = torch.cat([b_in, b_out[ok]])
    del a_in, b_in, a_out, b_out, ok, vblk
    keep = a != b
    a, b = a[keep], b[keep]
    lo_v = torch.minimum(a, b)
    hi_v = torch.maximum(a, b)
    del a, b, keep
    key = torch.unique(lo_v * N + hi_v)
    del lo_v, hi_v
    lo_v = key // N
    hi_v = key % N
    del key
    # converter relabelling inside each graph: (degree, id) descending
    deg = torch.bincount(lo_v, minlength=N) + torch.bincount(hi_v, minlength=N)
    vgraph = torch.repeat_interleave(torch.arange(G, device=dev), ns_t)
    local = torch.arange(N, device=dev) - goff[vgraph]
    skey = (vgraph << 42) | (((1 << 21) - 1 - deg) << 20) | ((1 << 20) - 1 - local)
    order = torch.argsort(skey)
    del skey, local
    rank = torch.empty_like(order)
    rank[order] = torch.arange(N, device=dev)
    new_local = rank - goff[vgraph]
    del rank, order
    n_new = torch.bincount(vgraph[deg > 0], minlength=G)
    new_off = torch.zeros(G + 1, dtype=torch.int64, device=dev)
    new_off[1:] = torch.cumsum(n_new, 0)
    fid = new_off[vgraph] + new_local            # isolated vertices sort last in their graph
    del new_local, vgraph, deg
    Nn = int(new_off[-1])
    a = fid[lo_v]
    b = fid[hi_v]
    del lo_v, hi_v, fid
    rows = torch.cat([a, b])
    cols = torch.cat([b, a])
    del a, b
    key = torch.sort(rows * Nn + cols).values
    del rows, cols
    rows = key // Nn
    cols = key % Nn
    del key
    counts = torch.bincount(rows, minlength=Nn)
    del rows
    indices = torch.zeros(Nn + 1, dtype=torch.int64, device=dev)
    indices[1:] = torch.cumsum(counts, 0)
    del counts
    cgraph = torch.repeat_interleave(torch.arange(G, device=dev), n_new)
    adj = (cols - new_off[cgraph[cols]]).to(torch.int32)
    del cols, cgraph
    voff = new_off.cpu().numpy().astype(np.int32)
    return voff, indices.to(torch.int32), adj


def unpack(voff, indices, adj):
    """Per-graph (indices, adj) numpy pairs of a packed batch (host arrays)."""
    out = []
    for g in range(len(voff) - 1):
        a, b = int(voff[g]), int(voff[g + 1])
        out.append(((indices[a:b + 1] - indices[a]).astype(np.int32), np.ascontiguousarray(adj[indices[a]:indices[b]])))
    return out
