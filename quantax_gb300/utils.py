"""Host-side helpers of the reference's utils package that the optimisation loop uses.

DataTracer records a scalar per step against a time axis (quantax/utils/data.py:8-147), the
quantity the time-stepping drivers append their energies, variances and step sizes to.
"""
from __future__ import annotations

from numbers import Number
from pathlib import Path
from typing import BinaryIO, Optional, Union

import numpy as np


class DataTracer:
    """A growing series of values with the time of each (data.py:8-66)."""

    def __init__(self):
        self._data_array = np.array([])
        self._time_array = np.array([])

    @property
    def data(self) -> np.ndarray:
        return self._data_array

    @property
    def time(self) -> np.ndarray:
        return self._time_array

    def append(self, data: Number, time: Optional[float] = None) -> None:
        """Append a value; the time defaults to the last time + 1 (0 for the first value)."""
        self._data_array = np.append(self._data_array, data)
        if time is None:
            time = 0 if self._time_array.size == 0 else self._time_array[-1] + 1
        self._time_array = np.append(self._time_array, time)

    def __getitem__(self, idx):
        return self._data_array[idx]

    def __array__(self, dtype=None, copy=None):
        return self.data if dtype is None else self.data.astype(dtype)

    def __len__(self) -> int:
        return self._data_array.size

    def __repr__(self):
        return self.data.__repr__()

    def mean(self) -> Number:
        return np.mean(self.data)

    def uncertainty(self) -> Optional[Number]:
        """Standard error of the mean, sqrt(sum |x - mean|^2 / (n (n - 1))); None below 2 values."""
        n = self.data.size
        if n < 2:
            return None
        diff = np.abs(self.data - self.mean()) ** 2
        return np.sqrt(np.sum(diff) / n / (n - 1))

    def save(self, file: Union[str, Path, BinaryIO]) -> None:
        np.save(file, self._data_array)

    def save_time(self, file: Union[str, Path, BinaryIO]) -> None:
        np.save(file, self._time_array)

    def batched(self, start: Optional[int] = None, end: Optional[int] = None, batch: int = 1):
        """(time, data) of [start, end) averaged over consecutive groups of `batch` values, the
        points plot() draws; a trailing partial group is dropped."""
        time = self._time_array[start:end]
        data = self._data_array[start:end]
        extra = data.size % batch
        if extra > 0:
            time, data = time[:-extra], data[:-extra]
        if data.size == 0:
            return time, data
        return time.reshape(-1, batch).mean(axis=1), data.reshape(-1, batch).mean(axis=1)

    def plot(self, start: Optional[int] = None, end: Optional[int] = None, batch: int = 1, logx: bool = False,
             logy: bool = False, baseline: Optional[Number] = None) -> None:
        """Plot the batched series with matplotlib (data.py:78-147); with logy and a baseline the
        relative error |data - baseline| / |baseline| is drawn, else a dashed line at baseline."""
        import matplotlib.pyplot as plt

        time, data = self.batched(start, end, batch)
        if data.size == 0:
            return
        if baseline is not None:
            if logy:
                data = (data - baseline) / abs(baseline)
            else:
                plt.hlines(baseline, xmin=time[0], xmax=time[-1], colors="k", linestyles="dashed")
        if logx and not logy:
            plt.semilogx(time, data)
        elif logy and not logx:
            plt.semilogy(time, data)
        elif logx and logy:
            plt.loglog(time, data)
        else:
            plt.plot(time, data)


def basis_states(n: int, nup: Optional[int] = None) -> np.ndarray:
    """Codes of the computational basis in ascending order (bit i set = site i up), all 2^n of
    them or the fixed-magnetisation sector with nup up spins (n <= 30)."""
    if n > 30:
        raise ValueError("a full basis is limited to n <= 30 sites")
    codes = np.arange(1 << n, dtype=np.int64)
    if nup is None:
        return codes
    count = np.zeros_like(codes)
    for i in range(n):
        count += (codes >> i) & 1
    return codes[count == nup]


def states_to_spins(states: np.ndarray, n: int) -> np.ndarray:
    """(len(states), n) int8 +-1 configurations of basis codes."""
    return ((((np.asarray(states)[:, None] >> np.arange(n)) & 1) * 2) - 1).astype(np.int8)
