"""In-memory stand-in for the h5py calls of the reference's gravitation/lib/simulation.py
(File, create_group, create_dataset, attrs, item access), persisted with pickle so that a
file written by one call can be read by the next.  Test infrastructure only: h5py is
absent on both hosts, so the HDF5 file format itself is not exercised."""
import os, pickle
import numpy as np

class _Group(dict):
    def __init__(self):
        super().__init__()
        self.attrs = {}
    def create_group(self, name):
        if name in self:
            raise ValueError('group %s exists' % name)
        self[name] = _Group()
        return self[name]
    def create_dataset(self, name, shape, dtype):
        self[name] = np.zeros(shape, dtype=np.dtype(dtype))
        return self[name]

class File(_Group):
    def __init__(self, fn, mode='r'):
        super().__init__()
        self._fn, self._mode = fn, mode
        if os.path.exists(fn):
            with open(fn, 'rb') as f:
                self.update(pickle.load(f))
        elif mode == 'r':
            raise OSError(fn)
    def close(self):
        if self._mode != 'r':
            with open(self._fn, 'wb') as f:
                pickle.dump(dict(self), f)
