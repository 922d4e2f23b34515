"""Linear pipeline of named steps (rubix/pipeline/abstract_pipeline.py:12-214,
linear_pipeline.py:10-187), run eagerly: the steps launch CUDA kernels, which
``jax.jit`` would not trace, so the composed expression is a plain Python loop.
"""

from __future__ import annotations

import functools
from typing import Callable, Dict, List


def bound_transformer(*args, **kwargs):
    """rubix/pipeline/transformer.py:7-21: bind leading args / kwargs to a step."""

    def wrap(kernel):
        if not args and not kwargs:
            return kernel
        f = functools.partial(kernel, *args, **kwargs)
        f.__name__ = getattr(kernel, "__name__", "step")
        return f

    return wrap


def step_names(cfg: dict) -> List[str]:
    """The transformer names of a linear pipeline config in run order ([] when the
    config is not a well-formed chain; ``LinearTransformerPipeline`` reports why)."""
    try:
        nodes = cfg["Transformers"]
        key = next(k for k, n in nodes.items() if n["depends_on"] is None)
        names = []
        while key is not None and len(names) <= len(nodes):
            names.append(nodes[key]["name"])
            key = next((k for k, n in nodes.items() if n["depends_on"] == key), None)
        return names
    except (KeyError, TypeError, AttributeError, StopIteration):
        return []


class LinearTransformerPipeline:
    """Steps registered by ``__name__`` and chained by the ``depends_on`` fields of the
    pipeline config (one start node, no branching)."""

    def __init__(self, cfg: dict, transformers: List[Callable]):
        self.config = cfg
        self.transformers: Dict[str, Callable] = {}
        self._pipeline: List[Callable] = []
        self._names: List[str] = []
        self.expression = None
        for t in transformers:
            self.register_transformer(t)
        self.assemble()

    def register_transformer(self, cls):
        """abstract_pipeline.py:65-82: the function's ``__name__`` is its key."""
        if cls.__name__ in self.transformers:
            raise ValueError("A transformer of this name is already present")
        self.transformers[cls.__name__] = cls

    @property
    def pipeline(self) -> dict:
        return dict(zip(self._names, self._pipeline))

    def assemble(self):
        self.build_pipeline()
        self.build_expression()

    def build_pipeline(self):
        """linear_pipeline.py:56-138 (same validation messages)."""
        if len(self.transformers) == 0:
            raise RuntimeError("No registered transformers present")
        nodes = self.config["Transformers"]
        deps = set()
        for key, node in nodes.items():
            if "name" not in node:
                raise ValueError("Each node of a pipeline must have a config node containing 'name'")
            if "args" not in node:
                raise ValueError("Config node must have a possibly empty args element")
            if "kwargs" not in node:
                raise ValueError("Config node must have a possible empty kwargs element")
            if "depends_on" not in node:
                raise ValueError("Config node must have a possibly 'null' valued node depends_on")
            dep = node["depends_on"]
            if dep is None:
                continue
            if dep in deps:
                raise ValueError(
                    "Dependencies must be unique in a linear pipeline as branching is not "
                    f"allowed. Found {dep} at least twice")
            deps.add(dep)
        start = [k for k, n in nodes.items() if n["depends_on"] is None]
        if len(start) > 1:
            raise ValueError("There can only be one starting point.")
        self._pipeline, self._names = [], []
        key = start[0]
        while key is not None:
            node = nodes[key]
            if node["name"] not in self.transformers:
                raise RuntimeError(f"Node '{node['name']}' not found in the config")
            self._pipeline.append(
                bound_transformer(*node["args"], **node["kwargs"])(self.transformers[node["name"]]))
            self._names.append(key)
            nxt = [k for k, n in nodes.items() if n["depends_on"] == key]
            key = nxt[0] if nxt else None

    def build_expression(self):
        pipeline = list(self._pipeline)

        def expr(data):
            res = data
            for f in pipeline:
                res = f(res)
            return res

        self.expression = expr

    def apply(self, *args, **kwargs):
        if len(args) == 0:
            raise ValueError("Cannot apply the pipeline to an empty list of arguments")
        return self.expression(*args, **kwargs)
