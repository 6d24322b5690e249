"""Solver callbacks, mirroring ffthompy/general/solver_pp.py:6-34.

The reference's CallBack recomputes B - Afun(x) after every CG iteration
(one extra operator application per iteration).  The fused GPU solver does
not stop between iterations, so CallBack.res_norm is filled from the
solver's recursive residual log (equal to ||B - A x_k|| in exact
arithmetic), at no extra cost.
"""


class CallBack:
    def __init__(self, **kwargs):
        self.__dict__.update(kwargs)
        self.iter = -1
        self.res_norm = []
        self.energy_norm = []

    def __call__(self, x):
        self.iter += 1
        res = self.B - self.A(x)
        self.res_norm.append(res.norm())

    def record_log(self, log):
        """Take the residual norms of a finished fused solve."""
        self.res_norm = [float(v) for v in log]
        self.iter = len(self.res_norm) - 1

    def __repr__(self):
        if not self.res_norm:
            return 'the results are not initialized yet'
        return '    iterations : %d\n    res_norm : %g\n' % (self.iter, self.res_norm[-1])
