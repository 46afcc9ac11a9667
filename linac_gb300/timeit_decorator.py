"""``@timeit``: prints the wall time of a call made with ``verbose=True``
(same behaviour and format as linac/timeit_decorator.py:8-22)."""
import functools
import time


def timeit(func):
    @functools.wraps(func)
    def wrapper_timeit(*args, **kwargs):
        start = time.time()
        value = func(*args, **kwargs)
        seconds = time.time() - start
        if kwargs.get("verbose") is True:
            ms = int(seconds * 1000) % 1000
            m, s = divmod(int(seconds), 60)
            h, m = divmod(m, 60)
            print("\rTime elapsed in %s: %d:%02d:%02d:%03d.                                        "
                  % (func.__name__, h, m, s, ms))
        return value
    return wrapper_timeit
