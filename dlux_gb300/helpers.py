"""Layer-dictionary helpers (dLux utils/helpers.py:93-230)."""

from __future__ import annotations

from collections import OrderedDict

__all__ = ["list2dictionary", "insert_layer", "remove_layer"]


def list2dictionary(list_in, ordered=True, allowed_types=()):
    """Key layers by class name (or an explicit (key, layer) tuple); repeats get _0, _1, ..."""
    names = []
    items = []
    for item in list_in:
        if isinstance(item, tuple):
            name, obj = item
        else:
            name, obj = item.__class__.__name__, item
        if allowed_types and not isinstance(obj, allowed_types):
            raise TypeError(f"Item {name} is not an allowed type, got {type(obj)}")
        names.append(name)
        items.append(obj)
    repeats = {n for n in names if names.count(n) > 1}
    counters = {n: 0 for n in repeats}
    for i, n in enumerate(names):
        if n in repeats:
            names[i] = f"{n}_{counters[n]}"
            counters[n] += 1
    out = OrderedDict() if ordered else {}
    for n, obj in zip(names, items):
        if " " in n:
            raise ValueError(f"Names cannot contain spaces, got {n}")
        out[n] = obj
    return out


def insert_layer(layers, layer, index, allowed_types=()):
    items = list(layers.items())
    items.insert(index, layer if isinstance(layer, tuple) else (layer.__class__.__name__, layer))
    return list2dictionary(items, True, allowed_types)


def remove_layer(layers, key):
    out = OrderedDict(layers)
    del out[key]
    return out
