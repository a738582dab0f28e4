"""The multicolour ordering restated in numpy, for the tests of
ocsl_set_ordering / ocsl_colour_pattern: the greedy colouring in natural
order, the colour-major permutation and the permuted system P A P^T, P b
(the reference's CSR layout, phantom columns kept after the real ones)."""
import numpy as np

from opencslsolver_gb300 import PHANTOM


def colour_order(row_ptr, column_index):
    """(perm, colours): row i gets the smallest colour none of its
    already-coloured neighbours has; rows numbered colour by colour,
    ascending within a colour; perm[new] = original row."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(column_index, dtype=np.uint64)
    n = rp.size - 1
    colour = np.full(n, -1, dtype=np.int64)
    for i in range(n):
        taken = set()
        for j in col[rp[i]:rp[i + 1]]:
            if j != PHANTOM and int(j) < i:
                taken.add(int(colour[int(j)]))
        c = 0
        while c in taken:
            c += 1
        colour[i] = c
    perm = np.argsort(colour, kind="stable").astype(np.int32)
    return perm, int(colour.max()) + 1 if n else 0


def permuted_pattern(row_ptr, column_index, perm):
    """(rp, col, slot) of the permuted pattern: row k is original row
    perm[k] with its columns renumbered and sorted, phantoms last;
    slot[new entry] = the original entry."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(column_index, dtype=np.uint64)
    n = rp.size - 1
    inv = np.empty(n, dtype=np.int64)
    inv[perm] = np.arange(n)
    new_rp = np.zeros(n + 1, dtype=np.uint64)
    new_col, slot = [], []
    for k in range(n):
        i = int(perm[k])
        q = np.arange(rp[i], rp[i + 1])
        real = col[q] != PHANTOM
        cols = inv[col[q][real].astype(np.int64)]
        order = np.argsort(cols, kind="stable")
        new_col.extend(cols[order].astype(np.uint64))
        slot.extend(q[real][order])
        for qq in q[~real]:
            new_col.append(PHANTOM)
            slot.append(qq)
        new_rp[k + 1] = len(new_col)
    return new_rp, np.asarray(new_col, dtype=np.uint64), np.asarray(slot, dtype=np.int64)


def permuted_system(s, perm):
    """(rp, col, value, b) of P A P^T, P b."""
    rp, col, slot = permuted_pattern(s.row_ptr, s.column_index, perm)
    return rp, col, np.asarray(s.value)[slot], np.asarray(s.b)[perm]
