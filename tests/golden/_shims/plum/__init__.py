"""Test-only stand-in for the plum features CoLA uses: ``dispatch`` (with ``precedence=`` and
``cond=``), ``dispatch.abstract`` and ``parametric``.

Methods register per (module, function name).  A call binds the arguments against each method's
signature (after applying the abstract signature's defaults), keeps the methods whose annotations
accept the arguments and whose ``cond`` holds, drops any method another candidate strictly
specialises, and breaks remaining ties by precedence."""
import inspect
import types
import typing

_FUNCTIONS = {}


def _accepts(value, ann):
    if ann is inspect.Parameter.empty or ann is typing.Any:
        return True
    origin = typing.get_origin(ann)
    if origin is typing.Union or isinstance(ann, types.UnionType):
        return any(_accepts(value, a) for a in typing.get_args(ann))
    if ann is typing.Callable or (origin is not None and origin.__module__ == "collections.abc"):
        return callable(value)
    if origin is not None:
        ann = origin
    try:
        return isinstance(value, ann)
    except TypeError:
        return True


def _classes(ann):
    if ann is inspect.Parameter.empty or ann is typing.Any:
        return [object]
    origin = typing.get_origin(ann)
    if origin is typing.Union or isinstance(ann, types.UnionType):
        return [c for a in typing.get_args(ann) for c in _classes(a)]
    if ann is typing.Callable or (origin is not None and origin.__module__ == "collections.abc"):
        return [object]
    return [origin or ann]


def _narrower_or_equal(a, b):
    return all(any(issubclass(x, y) for y in _classes(b)) for x in _classes(a))


class _Method:
    def __init__(self, fn, precedence, cond):
        self.fn, self.precedence, self.cond = fn, precedence, cond
        self.signature = inspect.signature(fn)
        self.params = list(self.signature.parameters.values())


def _strictly_more_specific(m1, m2):
    pairs = list(zip(m1.params, m2.params))
    return (all(_narrower_or_equal(p.annotation, q.annotation) for p, q in pairs)
            and not all(_narrower_or_equal(q.annotation, p.annotation) for p, q in pairs))


class _Function:
    def __init__(self, name):
        self.name, self.methods, self.abstract = name, [], None

    def __call__(self, *args, **kwargs):
        if self.abstract is not None:
            bound = self.abstract.bind(*args, **kwargs)
            bound.apply_defaults()
            args, kwargs = tuple(bound.arguments.values()), {}
        candidates = []
        for m in self.methods:
            try:
                bound = m.signature.bind(*args, **kwargs)
            except TypeError:
                continue
            bound.apply_defaults()
            ok = all(_accepts(bound.arguments[p.name], p.annotation) for p in m.params if p.name in bound.arguments)
            if ok and (m.cond is None or m.cond(*bound.args)):
                candidates.append((m, bound))
        if not candidates:
            raise NotImplementedError(f"no method of {self.name} for {tuple(type(a).__name__ for a in args)}")
        best = [c for c in candidates if not any(o is not c and _strictly_more_specific(o[0], c[0]) for o in candidates)]
        best.sort(key=lambda c: -c[0].precedence)
        m, bound = best[0]
        return m.fn(*bound.args, **bound.kwargs)


def _function_for(fn):
    f = _FUNCTIONS.setdefault((fn.__module__, fn.__name__), _Function(fn.__name__))
    f.__name__, f.__module__, f.__qualname__ = fn.__name__, fn.__module__, fn.__qualname__
    return f


class _Dispatcher:
    def __call__(self, fn=None, *, precedence=0, cond=None):
        def register(f):
            func = _function_for(f)
            func.methods.append(_Method(f, precedence, cond))
            return func
        return register(fn) if fn is not None else register

    def abstract(self, fn):
        func = _function_for(fn)
        func.abstract = inspect.signature(fn)
        return func


dispatch = _Dispatcher()


def parametric(cls):
    cache = {}

    def class_getitem(c, params):
        params = params if isinstance(params, tuple) else (params,)
        if params not in cache:
            name = f"{cls.__name__}[{','.join(getattr(p, '__name__', str(p)) for p in params)}]"
            cache[params] = type(name, (cls,), {})
        return cache[params]

    cls.__class_getitem__ = classmethod(class_getitem)
    return cls
