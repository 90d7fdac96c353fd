"""Minimal stand-in: the four helpers the reference imports."""
import itertools
from collections import defaultdict


def first(iterable, default=None):
    for v in iterable:
        return v
    if default is None:
        raise ValueError("first() was called on an empty iterable")
    return default


def take(n, iterable):
    return list(itertools.islice(iterable, n))


def windowed(seq, n):
    seq = list(seq)
    return [tuple(seq[i:i + n]) for i in range(0, max(len(seq) - n + 1, 0))]


def map_reduce(iterable, keyfunc, valuefunc=None, reducefunc=None):
    out = defaultdict(list)
    for item in iterable:
        out[keyfunc(item)].append(valuefunc(item) if valuefunc else item)
    if reducefunc is not None:
        return {k: reducefunc(v) for k, v in out.items()}
    return dict(out)
