"""Flattening of nested dict / list / tuple containers of tensors.

The counterpart of ``tree.ravel_pytree`` in matfree/backend/tree.py:15-20,
used at the same places (vectors and matvec outputs are pytrees,
matfree/funm.py:227-235, decomp.py:381-384).  Leaves are torch tensors; the
flat vector concatenates the leaves in insertion / index order.
"""

from __future__ import annotations

import torch


def _leaves(tree, out):
    if isinstance(tree, dict):
        for key in tree:
            _leaves(tree[key], out)
    elif isinstance(tree, (list, tuple)):
        for item in tree:
            _leaves(item, out)
    else:
        out.append(tree)
    return out


def _rebuild(tree, it):
    if isinstance(tree, dict):
        return type(tree)((key, _rebuild(val, it)) for key, val in tree.items())
    if isinstance(tree, tuple) and hasattr(tree, "_fields"):
        return type(tree)(*[_rebuild(v, it) for v in tree])
    if isinstance(tree, (list, tuple)):
        return type(tree)(_rebuild(v, it) for v in tree)
    return next(it)


def tree_leaves(tree):
    return _leaves(tree, [])


def ravel_pytree(tree):
    """Return (flat 1-D tensor, unravel) for a container of tensors.

    Leaves may be torch tensors or any DLPack-capable arrays (imported as
    torch views without a copy)."""
    from ._panel import as_tensor

    leaves = [as_tensor(leaf, "pytree leaf") for leaf in tree_leaves(tree)]
    if len(leaves) == 1 and not isinstance(tree, (dict, list, tuple)):
        leaf = leaves[0]
        shape = leaf.shape

        def unravel_single(flat):
            return flat.reshape(*flat.shape[:-1], *shape)

        return leaf.reshape(-1), unravel_single
    shapes = [leaf.shape for leaf in leaves]
    sizes = [leaf.numel() for leaf in leaves]
    flat = torch.cat([leaf.reshape(-1) for leaf in leaves]) if leaves else torch.zeros(0)

    def unravel(v):
        parts = torch.split(v, sizes, dim=-1)
        batch = v.shape[:-1]
        it = iter(p.reshape(*batch, *s) for p, s in zip(parts, shapes))
        return _rebuild(tree, it)

    return flat, unravel


def tree_map(fn, *trees):
    first = trees[0]
    if isinstance(first, dict):
        return type(first)((k, tree_map(fn, *[t[k] for t in trees])) for k in first)
    if isinstance(first, (list, tuple)):
        return type(first)(tree_map(fn, *items) for items in zip(*trees))
    return fn(*trees)
