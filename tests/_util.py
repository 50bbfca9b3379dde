"""Shared helpers for the tests: oracle factors -> C-ABI import arrays."""
import numpy as np


def tree_csr(tree):
    """node -> values CSR (ptr, idx) of an oracle or library tree."""
    lens = (np.asarray(tree.end) - np.asarray(tree.begin)).astype(np.int64)
    ptr = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(lens, out=ptr[1:])
    idx = np.concatenate([tree.perm[tree.begin[i]:tree.end[i]] for i in range(len(lens))])
    return ptr, idx.astype(np.int64)


def oracle_blocks(bfs):
    """Flatten oracle BF objects into the bf_factor_desc block arrays."""
    cols = dict(bf=[], stage=[], obs_out=[], src_out=[], obs_in=[], src_in=[], rows=[], cols=[],
                identity=[], data_off=[])
    chunks = []
    off = 0

    def add(i, st, b):
        nonlocal off
        cols["bf"].append(i)
        cols["stage"].append(st)
        cols["obs_out"].append(b.obs_out)
        cols["src_out"].append(b.src_out)
        cols["obs_in"].append(b.obs_in)
        cols["src_in"].append(b.src_in)
        if b.data is None:
            cols["rows"].append(0)
            cols["cols"].append(0)
            cols["identity"].append(1)
            cols["data_off"].append(off)
        else:
            r, c = b.data.shape
            cols["rows"].append(r)
            cols["cols"].append(c)
            cols["identity"].append(0)
            cols["data_off"].append(off)
            chunks.append(np.asarray(b.data, np.complex128).ravel(order="F"))
            off += r * c

    for i, bf in enumerate(bfs):
        for b in bf.Q:
            add(i, 0, b)
        for l, lvl in enumerate(bf.R):
            for b in lvl:
                add(i, l + 1, b)
        for b in bf.P:
            add(i, -1, b)
    out = {k: np.asarray(v) for k, v in cols.items()}
    out["data"] = np.concatenate(chunks) if chunks else np.zeros(1, np.complex128)
    return out


def import_oracle(bfs, n_rows, n_cols, tree_o, tree_s, ctx=None):
    import bfgpu
    d = oracle_blocks(bfs)
    return bfgpu.import_blocks(n_rows, n_cols, d["bf"], d["stage"], d["obs_out"], d["src_out"],
                               d["obs_in"], d["src_in"], d["rows"], d["cols"], d["identity"],
                               d["data_off"], d["data"], tree_csr(tree_o), tree_csr(tree_s), ctx)


def relerr(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b)))


def export_to_oracle(ex, tree_o, tree_s, k=0.0, tau=0.0):
    """bf_op_export_blocks arrays -> list of oracle BF objects (pointer-wired)."""
    from oracle import bfref as O
    nbf = int(ex["bf"].max()) + 1 if len(ex["bf"]) else 0
    per = [dict(Q=[], R={}, P=[]) for _ in range(nbf)]
    for b in range(len(ex["bf"])):
        f, st = int(ex["bf"][b]), int(ex["stage"][b])
        if ex["identity"][b]:
            data = None
        else:
            r, c, off = int(ex["rows"][b]), int(ex["cols"][b]), int(ex["data_off"][b])
            data = ex["data"][off:off + r * c].reshape((r, c), order="F")
        blk = O.Block(int(ex["obs_out"][b]), int(ex["src_out"][b]), int(ex["obs_in"][b]),
                      int(ex["src_in"][b]), data)
        if st == 0:
            per[f]["Q"].append(blk)
        elif st < 0:
            per[f]["P"].append(blk)
        else:
            per[f]["R"].setdefault(st, []).append(blk)
    out = []
    for f in range(nbf):
        d = per[f]
        R = [d["R"][l] for l in sorted(d["R"])]
        no = d["Q"][0].obs_out if d["Q"] else 0
        ns = d["P"][0].src_out if d["P"] else 0
        out.append(O.BF(d["Q"], R, d["P"], tree_o, tree_s, k, tau, no, ns).wire())
    return out


class CsrTree:
    """The part of the tree contract the oracle matvec uses (``values(node)``),
    from a node -> values CSR map (ptr, idx)."""

    def __init__(self, ptr, idx):
        self.ptr = np.asarray(ptr, np.int64)
        self.idx = np.asarray(idx, np.int64)

    def values(self, node):
        return self.idx[self.ptr[node]:self.ptr[node + 1]]


def oracle_apply(bfs, x, n_out, op="N"):
    """Oracle far-field product op(A) x over the BF list (reference-order flat
    matvec of each block, the materialised adjoint / transpose for "C" / "T")."""
    from oracle import bfref as O
    y = np.zeros(n_out, np.complex128)
    for bf in bfs:
        b = bf if op == "N" else O.adjoint_bf(bf, op)
        O.matvec_flat(b, x, y, 1.0, 1.0)
    return y
