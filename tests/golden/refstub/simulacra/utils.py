"""``simulacra.utils`` helpers used by the reference mesh path (stub)."""

import collections
import enum
import functools
import time

import numpy as np


class StrEnum(str, enum.Enum):
    def __str__(self):
        return str(self.value)

    def __repr__(self):
        return f"{self.__class__.__name__}.{self.name}"


def memoize(func):
    """Cache results keyed on the call arguments (as simulacra.utils.memoize)."""
    cache = {}

    @functools.wraps(func)
    def wrapper(*args, **kwargs):
        key = (args, tuple(sorted(kwargs.items())))
        try:
            return cache[key]
        except KeyError:
            value = func(*args, **kwargs)
            cache[key] = value
            return value
        except TypeError:  # unhashable argument
            return func(*args, **kwargs)

    return wrapper


def watched_memoize(watcher):
    def deco(func):
        return memoize(func)

    return deco


cached_property = functools.cached_property

NearestEntry = collections.namedtuple("NearestEntry", ("index", "value", "target"))


def find_nearest_entry(array, target):
    array = np.array(array)
    index = int(np.argmin(np.abs(array - target)))
    return NearestEntry(index, array[index], target)


def bytes_to_str(num):
    return f"{num} B"


def dict_to_arrays(d, key=None):
    keys = sorted(d.keys(), key=key)
    return np.array(keys), np.array([d[k] for k in keys])


class BlockTimer:
    def __enter__(self):
        self.start = time.perf_counter()
        self.proc_start = time.process_time()
        return self

    def __exit__(self, *exc):
        self.wall_time_elapsed = time.perf_counter() - self.start
        self.proc_time_elapsed = time.process_time() - self.proc_start


class LogManager:
    def __init__(self, *args, **kwargs):
        pass

    def __enter__(self):
        import logging

        return logging.getLogger("stub")

    def __exit__(self, *exc):
        pass


def table(headers, rows):
    return "\n".join([" | ".join(headers)] + [" | ".join(r) for r in rows])
