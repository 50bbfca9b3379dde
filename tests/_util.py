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
    return O.from_blocks(ex, tree_o, tree_s, k, tau)


def CsrTree(ptr, idx):
    """node -> values CSR map as an oracle tree (``values(node)``)."""
    from oracle import bfref as O
    return O.CsrTree(ptr, idx)


def oracle_apply(bfs, x, n_out, op="N"):
    """Oracle far-field product op(A) x over the BF list (reference-order flat
    matvec of each block, the materialised adjoint / transpose for "C" / "T")."""
    from oracle import bfref as O
    return O.apply_far(bfs, x, n_out, op)
