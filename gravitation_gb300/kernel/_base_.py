"""Stand-alone restatement of the reference's plugin interface ``universe_base``.

gravitation/kernel/_base_.py:31-177 defines the class every kernel derives from.  The
``gb1`` package imports ``universe_base`` relatively (``from .._base_ import
universe_base``): inside the reference tree that resolves to the reference's own
class; inside this repository it resolves to this file, so the same kernel package
runs in both places.  This file keeps the reference's interface -- names, argument
meaning, scaling, state machine and the SyntaxError it raises on misuse -- because
front-end code relies on exactly that; the code itself is written here.

  universe(t=0.0, T=1e3, G=6.6740831e-11, scale_m=1.0, scale_r=1.0,
           dtype='float32', threads=1, **kwargs)      (_base_.py:69-93)
    G is scaled once to G * scale_r**3 / scale_m unless scale_off=True
    unknown keyword arguments are kept in self._meta
  add_object(name=, r=[3], v=[3], m=, [scale_off])    (_base_.py:107-118)
    r and v are multiplied by scale_r, m by scale_m, unless scale_off
  start() -> start_kernel()                           (_base_.py:120-134)
  step()  -> step_stage1(); step_stage2(); step_stage3()   (_base_.py:136-161)
  stop()  -> stop_kernel()                            (_base_.py:163-177)
  iteration yields the point masses (_name, _r, _v, _a, _m)
"""

PREINIT, STARTED, STOPPED = 0, 1, 2


class _point_mass:
    """One body: name, position, velocity, acceleration (zeroed) and mass."""

    def __init__(self, name, r, v, m):
        self._name = name
        self._r = r
        self._v = v
        self._a = [0.0] * len(r)
        self._m = m

    def __str__(self):
        x, y, z = self._r
        vx, vy, vz = self._v
        return '%s | %.4e, %.4e, %.4e | %.4e, %.4e, %.4e' % (self._name, x, y, z, vx, vy, vz)

    def move(self, T):
        """Base stage 2 for one body: v = a*T + v, then r = v*T + r, then a = 0."""
        self._v[:] = [a * T + v for v, a in zip(self._v, self._a)]
        self._r[:] = [v * T + r for r, v in zip(self._r, self._v)]
        self._a[:] = [0.0] * len(self._a)


class universe_base:
    """Plugin base: state machine, scaling, default stage 2 (see module docstring)."""

    def __init__(self, t=0.0, T=1.0e3, G=6.6740831e-11, scale_m=1.0, scale_r=1.0,
                 dtype='float32', threads=1, **kwargs):
        self._scale_m = scale_m
        self._scale_r = scale_r
        self._t = t
        self._T = T
        scale_off = kwargs.pop('scale_off', False)
        self._G = G if scale_off else G * scale_r ** 3 / scale_m
        self._mass_list = []
        self._state = PREINIT
        self._dtype = dtype
        self._threads = threads
        self._meta = kwargs

    def __iter__(self):
        return iter(self._mass_list)

    def __len__(self):
        return len(self._mass_list)

    def __str__(self):
        return '\n'.join(str(pm) for pm in self._mass_list)

    def add_object(self, **kwargs):
        if self._state == STARTED:
            raise SyntaxError('simulation was started')
        if self._state == STOPPED:
            raise SyntaxError('simulation was stopped')
        if not kwargs.pop('scale_off', False):
            kwargs['r'][:] = [c * self._scale_r for c in kwargs['r']]
            kwargs['v'][:] = [c * self._scale_r for c in kwargs['v']]
            kwargs['m'] *= self._scale_m
        self._mass_list.append(_point_mass(**kwargs))

    def start(self):
        if self._state == STARTED:
            raise SyntaxError('simulation is running')
        if self._state == STOPPED:
            raise SyntaxError('simulation was stopped')
        self._state = STARTED
        self.start_kernel()

    def start_kernel(self):
        pass

    def step(self):
        if self._state == PREINIT:
            raise SyntaxError('simulation was not started')
        if self._state == STOPPED:
            raise SyntaxError('simulation was stopped')
        self.step_stage1()
        self.step_stage2()
        self.step_stage3()

    def step_stage1(self):
        raise NotImplementedError()

    def step_stage2(self):
        for pm in self._mass_list:
            pm.move(self._T)

    def step_stage3(self):
        self._t += self._T

    def stop(self):
        if self._state == PREINIT:
            raise SyntaxError('simulation was not started')
        if self._state == STOPPED:
            raise SyntaxError('simulation was stopped before')
        self._state = STOPPED
        self.stop_kernel()

    def stop_kernel(self):
        pass
