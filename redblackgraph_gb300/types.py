"""Result and colour types (the reference's redblackgraph/types/{transitive_closure,color,ordering}.py)."""
from dataclasses import dataclass
from typing import Dict, Sequence

import numpy as np


@dataclass
class TransitiveClosure:
    W: np.ndarray
    diameter: int


class Color:
    RED = -1
    BLACK = 1


@dataclass
class Ordering:
    """A permuted matrix, the permutation (p[new] = old) and component sizes (ordering.py:5-9)."""
    A: Sequence[Sequence[int]]
    label_permutation: Sequence[int]
    components: Dict[int, int]
