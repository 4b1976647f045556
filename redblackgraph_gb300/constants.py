"""Red/black identities (the reference's redblackgraph/constants.py:71-105).

BLACK_ONE (1) is the multiplicative identity for odd (female) values, RED_ONE (-1) for even
(male) values; unsigned dtypes store RED_ONE as the dtype's maximum.
"""
import numpy as np

BLACK_ONE = 1
RED_ONE = -1


def red_one_for_dtype(dtype):
    dt = np.dtype(dtype)
    return int(np.iinfo(dt).max) if dt.kind == "u" else RED_ONE


def black_one_for_dtype(dtype):
    return BLACK_ONE


def is_red_one(value, dtype=None) -> bool:
    if dtype is not None and np.dtype(dtype).kind == "u":
        return int(value) == int(np.iinfo(np.dtype(dtype)).max)
    return int(value) == RED_ONE


def is_black_one(value, dtype=None) -> bool:
    return int(value) == BLACK_ONE
