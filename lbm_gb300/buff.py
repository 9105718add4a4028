"""Observable buffer with moving averages and a convergence test.

Same interface and arithmetic as lbm/src/utils/buff.py:8-77 (``add``,
``f_avg``, ``p_avg``, ``mv_avg``; ``obs``, ``obs_cv``), but the histories are
preallocated arrays grown by doubling instead of ``np.append`` at every call,
so a long run costs O(n) copies instead of O(n^2).  ``p_avg`` sums the same
slices with ``np.sum`` and therefore returns the same values.

``add_chunk`` does ``add`` + ``mv_avg`` for a whole array of values at once
on the GPU (``lbm_mv_avg_chunk``: the window sums of every add in parallel,
in NumPy's summation order), which removes the O(n) host sums per iteration
that make long runs quadratic; the histories then stay on the device until
a host method needs them.
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
        self._to_host()
        return self._buff.view()

    @property
    def avg1_buff(self):
        self._to_host()
        return self._avg1.view()

    @property
    def avg2_buff(self):
        self._to_host()
        return self._avg2.view()

    @property
    def avg3_buff(self):
        self._to_host()
        return self._avg3.view()

    # ---- device histories (add_chunk)
    _hist = None      # torch [4, cap] on the device while the GPU holds the histories
    _state = None     # torch int32 [2]: convergence counter and flag

    def _to_device(self, need):
        import torch
        if self._hist is not None and self._hist.shape[1] >= need:
            return
        cap = max(need, 2 * (self._hist.shape[1] if self._hist is not None else 0), 4096)
        hist = torch.zeros((4, cap), dtype=torch.float64, device="cuda")
        if self._hist is not None:
            hist[:, :self._hist.shape[1]] = self._hist
        else:
            n = self.it + 2
            for k, ser in enumerate((self._buff, self._avg1, self._avg2, self._avg3)):
                hist[k, :n] = torch.from_numpy(ser.view().copy()).to("cuda")
            self._state = torch.tensor([self.obs_cv_cnt, int(self.obs_cv)], dtype=torch.int32,
                                       device="cuda")
        self._hist = hist

    def _to_host(self):
        """Bring the histories back after add_chunk (for the host methods)."""
        if self._hist is None:
            return
        n = self.it + 2
        h = self._hist[:, :n].cpu().numpy()
        self._buff, self._avg1, self._avg2, self._avg3 = (_Series(h[k]) for k in range(4))
        self._hist = None
        self._state = None

    def add_chunk(self, values):
        """``add(v); mv_avg()`` for each value, in order, on the GPU.

        Returns (obs, growth, cv): what each ``mv_avg`` returned and the
        ``obs_cv`` flag after it, as arrays; equal bit for bit to the host
        calls.
        """
        import torch
        from . import _lib
        vals = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        n = len(vals)
        if n == 0:
            return np.zeros(0), np.zeros(0), np.zeros(0, bool)
        k0 = self.it
        self._to_device(k0 + n + 2)
        hist = self._hist
        hist[0, k0 + 2:k0 + 2 + n] = torch.from_numpy(vals).to("cuda")
        out = torch.empty((2, n), dtype=torch.float64, device="cuda")
        cv = torch.empty(n, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        _lib.call("lbm_mv_avg_chunk", hist.data_ptr(), hist.shape[1], k0, n, float(self.dt),
                  float(self.obs_cv_ct), int(self.obs_cv_nb), self._state.data_ptr(),
                  out[0].data_ptr(), out[1].data_ptr(), cv.data_ptr(), stream)
        o = out.cpu().numpy()
        c = cv.cpu().numpy().astype(bool)
        st = self._state.cpu().numpy()
        self.it += n
        self.obs = o[0, -1]
        self.obs_cv_cnt = int(st[0])
        self.obs_cv = bool(st[1])
        return o[0].copy(), o[1].copy(), c

    def add(self, value):
        self._to_host()
        self._buff.append(value)
        self.it += 1

    def f_avg(self):
        self._to_host()
        b = self._buff.view()
        return np.sum(b) / len(b)

    def p_avg(self, buff, i, j):
        return np.sum(buff[i:j]) / (float(j - i + 1))

    def mv_avg(self):
        self._to_host()
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
