"""Observable buffer with moving averages and a convergence test.

Same interface and arithmetic as lbm/src/utils/buff.py:8-77 (``add``,
``f_avg``, ``p_avg``, ``mv_avg``; ``obs``, ``obs_cv``), but the histories are
preallocated arrays grown by doubling instead of ``np.append`` at every call,
so a long run costs O(n) copies instead of O(n^2).  ``p_avg`` sums the same
slices with ``np.sum`` and therefore returns the same values.
"""
import math

import numpy as np


class _Series:
    """Append-only float64 array with amortised O(1) append."""

    def __init__(self, initial):
        self._a = np.zeros(max(16, 2 * len(initial)))
        self._n = len(initial)
        self._a[:self._n] = initial

    def append(self, v):
        if self._n == len(self._a):
            b = np.zeros(2 * len(self._a))
            b[:self._n] = self._a[:self._n]
            self._a = b
        self._a[self._n] = v
        self._n += 1

    def view(self):
        return self._a[:self._n]

    def __len__(self):
        return self._n


class buff:
    def __init__(self, name, dt, obs_cv_ct, obs_cv_nb, output_dir):
        self.name = name
        self._buff = _Series(np.zeros([2]))
        self._avg1 = _Series(np.zeros([2]))
        self._avg2 = _Series(np.zeros([2]))
        self._avg3 = _Series(np.zeros([2]))
        self.it = 0
        self.dt = dt
        self.output_dir = output_dir
        self.freq = 1.0
        self.obs = 0.0
        self.obs_cv_ct = obs_cv_ct
        self.obs_cv_nb = obs_cv_nb
        self.obs_cv_cnt = 0
        self.obs_cv = False

    # Read-only views with the reference attribute names.
    @property
    def buff(self):
        return self._buff.view()

    @property
    def avg1_buff(self):
        return self._avg1.view()

    @property
    def avg2_buff(self):
        return self._avg2.view()

    @property
    def avg3_buff(self):
        return self._avg3.view()

    def add(self, value):
        self._buff.append(value)
        self.it += 1

    def f_avg(self):
        b = self._buff.view()
        return np.sum(b) / len(b)

    def p_avg(self, buff, i, j):
        return np.sum(buff[i:j]) / (float(j - i + 1))

    def mv_avg(self):
        self.f_avg()
        it_s = math.floor(self.it * 4 / 5)
        it_e = self.it
        self.obs = self.p_avg(self._buff.view(), it_s, it_e)
        self._avg1.append(self.obs)
        self.obs = self.p_avg(self._avg1.view(), it_s, it_e)
        self._avg2.append(self.obs)
        self.obs = self.p_avg(self._avg2.view(), it_s, it_e)
        self._avg3.append(self.obs)
        self.obs = self.p_avg(self._avg3.view(), it_s, it_e)

        growth = 0.0
        if self.it > 10:
            a3 = self._avg3.view()
            db = a3[it_e] - a3[it_s]
            growth = db / ((it_e - it_s + 1) * self.dt)
            if abs(growth) < self.obs_cv_ct:
                self.obs_cv_cnt += 1
            else:
                self.obs_cv_cnt = 0
            if self.obs_cv_cnt > self.obs_cv_nb:
                self.obs_cv = True
        return self.obs, growth
