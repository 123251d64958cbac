"""NumPy backend of the Veros operators: in-place update, Python for-loop."""
import numpy


class _Index:
    def __getitem__(self, idx):
        return idx


at = _Index()


def update(arr, idx, value):
    arr[idx] = value
    return arr


def for_loop(lower, upper, body, init_val):
    val = init_val
    for i in range(lower, upper):
        val = body(i, val)
    return val
