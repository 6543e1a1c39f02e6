"""Host-side inputs to the likelihood path: root prior, error model, gamma
categories.

* `RootPrior` mirrors `root_equilibrium_distribution`
  (src/root_equilibrium_distribution.cpp:15-87). `compute(j)` returns a
  C float (src/root_equilibrium_distribution.h:40), so `vector()` returns
  float32-rounded values widened to float64, indexed by root-vector index j.
* `ErrorModel` mirrors `error_model` (src/error_model.cpp:11-109): rows of
  probabilities over count deviations {-1, 0, +1}, missing rows copy the
  previous row, `get_probs` clamps to the last row.
* `discrete_gamma` gives the median-based equal-probability discretisation
  of a Gamma(alpha, beta=alpha) rate (Yang 1994), as `get_gamma` does
  (src/gamma.cpp:15-52, 225-241): r_k = median of bin k, rescaled to mean 1;
  every category has probability 1/K. The quantile here is computed to full
  double precision; the reference's table-free AS91 routine stops at a
  relative tolerance of 5e-7, so multipliers agree to about 1e-6.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence

import numpy as np


class RootPrior:
    def __init__(self, freq: Sequence[float]):
        self._freq = np.asarray(freq, dtype=np.float64)

    @classmethod
    def uniform(cls, max_size: int) -> "RootPrior":
        # vectorized distribution 0..max_size-1, each with count 1
        pct = np.float32(1.0) / np.float32(max_size)
        return cls([float(pct)] * max_size)

    @classmethod
    def from_rootdist(cls, rootdist: Dict[int, int]) -> "RootPrior":
        if not rootdist:
            raise ValueError("No root distribution specified")
        total = sum(rootdist.values())
        mx = max(rootdist) + 1
        return cls([float(np.float32(rootdist.get(i, 0)) / np.float32(total)) for i in range(mx)])

    @classmethod
    def poisson(cls, lam: float, num_values: int) -> "RootPrior":
        freq: List[float] = []
        n_vec = 0
        i = 0
        while n_vec < num_values:
            pct = poisspdf(i, lam)
            n_vec += int(math.ceil(pct * num_values)) if pct * num_values > 0 else 0
            freq.append(pct)
            i += 1
        for _ in range(5):
            freq.append(poisspdf(len(freq), lam))
        return cls([float(np.float32(p)) for p in freq])

    def compute(self, j: int) -> float:
        return float(self._freq[j]) if 0 <= j < len(self._freq) else 0.0

    def vector(self, n: Optional[int] = None) -> np.ndarray:
        if n is None:
            return self._freq.copy()
        out = np.zeros(n, dtype=np.float64)
        k = min(n, len(self._freq))
        out[:k] = self._freq[:k]
        return out


def poisspdf(x: int, lam: float) -> float:
    """Poisson pmf in the reference's log form (src/poisson.cpp:21-24)."""
    return math.exp(x * math.log(lam) - math.lgamma(x + 1) - lam)


class ErrorModel:
    def __init__(self, deviations: Sequence[int] = (-1, 0, 1)):
        self.deviations = list(deviations)
        self.rows: List[List[float]] = []
        self.max_family_size = 0

    def set_probabilities(self, fam_size: int, probs: Sequence[float]) -> None:
        probs = list(probs)
        if (fam_size == 0 or not self.rows) and abs(probs[0]) > 0.0:
            raise ValueError("Cannot have a non-zero probability for family size 0 for negative deviation")
        if abs(sum(probs) - 1.0) > 0.01:
            raise ValueError("Sum of probabilities must be equal to one")
        if not self.rows:
            self.rows.append(probs)
        if len(self.rows) <= fam_size:
            self.rows.extend([list(self.rows[-1]) for _ in range(fam_size + 1 - len(self.rows))])
        self.rows[fam_size] = probs

    def get_probs(self, fam_size: int) -> List[float]:
        return self.rows[min(fam_size, len(self.rows) - 1)]

    def table(self) -> np.ndarray:
        return np.asarray(self.rows, dtype=np.float64)

    def get_epsilons(self) -> List[float]:
        return sorted({r[-1] for r in self.rows})

    def replace_epsilons(self, new_eps: Dict[float, float]) -> None:
        """src/error_model.cpp:79-109"""
        def near(x, y):
            return abs(x - y) <= 0.01 * abs(x)
        vec = list(self.rows[0])
        for old, new in sorted(new_eps.items()):
            if near(old, vec[-1]):
                vec[-1] = new
                vec[1] = 1 - new
                self.set_probabilities(0, vec)
        for i in range(1, len(self.rows)):
            vec = list(self.rows[i])
            for old, new in sorted(new_eps.items()):
                if near(old, vec[-1]):
                    vec[-1] = new
                    vec[0] = new
                    vec[1] = 1 - 2 * new
                    self.set_probabilities(i, vec)

    @classmethod
    def symmetric(cls, epsilon: float, max_count: int) -> "ErrorModel":
        """Row 0 = {0, 1-eps, eps}, rows >= 1 = {eps, 1-2eps, eps}."""
        em = cls()
        em.set_probabilities(0, [0.0, 1.0 - epsilon, epsilon])
        em.set_probabilities(max(max_count, 1), [epsilon, 1.0 - 2 * epsilon, epsilon])
        for i in range(1, max(max_count, 1)):
            em.rows[i] = [epsilon, 1.0 - 2 * epsilon, epsilon]
        em.max_family_size = max_count
        return em

    @classmethod
    def parse(cls, text: str) -> "ErrorModel":
        """The error-model file format (src/io.cpp:228-274)."""
        em = cls()
        for line in text.splitlines():
            if line.startswith("max"):
                em.max_family_size = int(line.split(":")[1].strip())
            elif line.startswith("cnt"):
                em.deviations = [int(x) for x in line.split()[1:]]
            elif line.strip():
                tok = line.split()
                em.set_probabilities(int(tok[0]), [float(x) for x in tok[1:]])
        return em


def discrete_gamma(alpha: float, K: int) -> (List[float], List[float]):
    """(category probabilities, rate multipliers) for K median categories of
    a mean-1 Gamma(alpha) (get_gamma, src/gamma.cpp:225-241), computed by the
    library's restatement of the reference's AS 91 / AS 32 / AS 70 routines
    so that the multipliers match the reference's bit for bit."""
    if K <= 1:
        return [1.0], [1.0]
    import ctypes
    from . import _lib
    probs = (ctypes.c_double * K)()
    mult = (ctypes.c_double * K)()
    rc = _lib.load().cafe_discrete_gamma(K, float(alpha), ctypes.addressof(probs), ctypes.addressof(mult))
    if rc != 0:
        raise ValueError(f"discrete gamma needs alpha > 0 (got {alpha})")
    return list(probs), list(mult)
