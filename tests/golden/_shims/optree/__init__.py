"""Test-only stand-in for the optree calls CoLA makes (register/flatten/unflatten/structure).

Registered classes flatten through their own tree_flatten / tree_unflatten methods; tuples,
lists and dicts recurse; everything else is a leaf."""
_REGISTERED = []


def register_pytree_node_class(cls, namespace=None):
    _REGISTERED.append(cls)
    return cls


def _is_node(v):
    return hasattr(v, "tree_flatten") and any(isinstance(v, c) for c in _REGISTERED)


class TreeSpec:
    def __init__(self, kind, meta, children):
        self.kind, self.meta, self.children = kind, meta, children


def _flatten(v, leaves):
    if v is None:
        return TreeSpec("none", None, [])
    if isinstance(v, (tuple, list)):
        return TreeSpec(type(v), None, [_flatten(c, leaves) for c in v])
    if isinstance(v, dict):
        keys = sorted(v)
        return TreeSpec("dict", keys, [_flatten(v[k], leaves) for k in keys])
    if _is_node(v):
        children, aux = v.tree_flatten()
        return TreeSpec("node", (type(v), aux), [_flatten(c, leaves) for c in children])
    leaves.append(v)
    return TreeSpec("leaf", None, [])


def tree_flatten(value, namespace=None, **kwargs):
    leaves = []
    return leaves, _flatten(value, leaves)


def tree_structure(value, namespace=None, **kwargs):
    return tree_flatten(value)[1]


def treespec_is_leaf(spec):
    return spec.kind == "leaf"


def _unflatten(spec, it):
    if spec.kind == "leaf":
        return next(it)
    if spec.kind == "none":
        return None
    kids = [_unflatten(c, it) for c in spec.children]
    if spec.kind == "dict":
        return dict(zip(spec.meta, kids))
    if spec.kind == "node":
        cls, aux = spec.meta
        return cls.tree_unflatten(aux, kids)
    return spec.kind(kids)


def tree_unflatten(spec, leaves):
    return _unflatten(spec, iter(list(leaves)))
