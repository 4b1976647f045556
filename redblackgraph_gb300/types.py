"""Result and colour types (the reference's redblackgraph/types/{transitive_closure,color}.py)."""
from dataclasses import dataclass

import numpy as np


@dataclass
class TransitiveClosure:
    W: np.ndarray
    diameter: int


class Color:
    RED = -1
    BLACK = 1
