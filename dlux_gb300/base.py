"""Immutable-object helpers mirroring the zodiax ``Base`` API used across dLux.

dLux objects are immutable pytrees updated through ``.set/.get/.add/.multiply``
with dotted paths (e.g. ``optics.set("layers.aperture.coefficients", c)``,
``instruments.py:249``). This class gives the same methods over plain Python
attributes; each update returns a shallow copy.
"""

from __future__ import annotations

import copy
from collections import OrderedDict

import torch


def _split(path):
    return path.split(".") if isinstance(path, str) else list(path)


def _get_child(obj, key):
    if isinstance(obj, (dict, OrderedDict)):
        return obj[key]
    if isinstance(obj, (list, tuple)):
        return obj[int(key)]
    return object.__getattribute__(obj, key) if hasattr(type(obj), "__dict__") and \
        key in getattr(obj, "__dict__", {}) else getattr(obj, key)


def _with_child(obj, key, value):
    if isinstance(obj, (dict, OrderedDict)):
        new = obj.copy()
        new[key] = value
        return new
    if isinstance(obj, list):
        new = list(obj)
        new[int(key)] = value
        return new
    if isinstance(obj, tuple):
        new = list(obj)
        new[int(key)] = value
        return tuple(new)
    new = copy.copy(obj)
    object.__setattr__(new, key, value)
    return new


def _set_path(obj, parts, value):
    if len(parts) == 1:
        return _with_child(obj, parts[0], value)
    child = _get_child(obj, parts[0])
    return _with_child(obj, parts[0], _set_path(child, parts[1:], value))


class Base:
    """zodiax-style immutable base class."""

    def get(self, path):
        obj = self
        for p in _split(path):
            obj = _get_child(obj, p)
        return obj

    def set(self, paths=None, values=None, **kwargs):
        if paths is None and not kwargs:
            raise TypeError("set() needs a path and a value, or keyword updates")
        if kwargs:
            obj = self
            for k, v in kwargs.items():
                obj = obj.set(k, v)
            return obj
        if isinstance(paths, (list, tuple)) and not isinstance(paths, str) and \
                all(isinstance(p, str) for p in paths) and isinstance(values, (list, tuple)):
            obj = self
            for p, v in zip(paths, values):
                obj = obj.set(p, v)
            return obj
        return _set_path(self, _split(paths), values)

    def add(self, path, value):
        return self.set(path, self.get(path) + value)

    def multiply(self, path, value):
        return self.set(path, self.get(path) * value)

    def divide(self, path, value):
        return self.set(path, self.get(path) / value)

    def min(self, path, value):
        return self.set(path, torch.minimum(self.get(path), torch.as_tensor(value)))
