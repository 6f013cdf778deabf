"""Particle container on the GPU, mirroring tupan/particles/body.py.

Structure-of-arrays float64 torch tensors on one CUDA device, with the
reference's attribute names (body.py:26-39: mass, eps2, rx, ry, rz, vx, vy,
vz, time, nstep, tstep), `register_auxiliary_attribute` for kernel outputs
(allparticles.py:64-76), slicing, `copy()`, the `set_*` force methods
(body.py:324-361) and the energy diagnostics (body.py:259-321).  Everything
stays resident in HBM between kernel calls.
"""
import numpy as np
import torch

from ._native import psum
from .lib import extensions

REAL_ATTRS = ("mass", "eps2", "rx", "ry", "rz", "vx", "vy", "vz", "time", "tstep")
INT_ATTRS = ("id", "nstep")


class ParticleSystem(object):
    """n particles; every attribute is a length-n tensor on `device`."""

    include_pn_corrections = False
    t_curr = 0.0

    def __init__(self, n=0, device=None, **arrays):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
        self.__dict__["_device"] = torch.device(device)
        self.n = int(n)
        for a in REAL_ATTRS:
            setattr(self, a, torch.zeros(self.n, dtype=torch.float64, device=self._device))
        self.id = torch.arange(self.n, dtype=torch.int64, device=self._device)
        self.nstep = torch.zeros(self.n, dtype=torch.int64, device=self._device)
        for k, v in arrays.items():
            self.set_array(k, v)

    # ---- construction helpers -------------------------------------------------
    @classmethod
    def from_arrays(cls, device=None, **arrays):
        n = len(next(iter(arrays.values())))
        return cls(n, device=device, **arrays)

    def set_array(self, name, value):
        t = torch.as_tensor(np.asarray(value) if not isinstance(value, torch.Tensor) else value)
        dtype = torch.int64 if name in INT_ATTRS else torch.float64
        t = t.to(device=self._device, dtype=dtype).contiguous()
        if t.shape != (self.n,):
            raise ValueError("%s must have shape (%d,)" % (name, self.n))
        setattr(self, name, t)

    def register_auxiliary_attribute(self, attr, sctype):
        if attr in self.__dict__:
            raise ValueError("'{0}' is already a registered attribute.".format(attr))
        dtype = torch.float64 if sctype == "real" else torch.int64
        setattr(self, attr, torch.zeros(self.n, dtype=dtype, device=self._device))

    def _arrays(self):
        return {k: v for k, v in self.__dict__.items() if isinstance(v, torch.Tensor)}

    def copy(self):
        new = ParticleSystem.__new__(ParticleSystem)
        new.__dict__["_device"] = self._device
        new.n = self.n
        for k, v in self._arrays().items():
            setattr(new, k, v.clone())
        return new

    def append(self, other):
        """Concatenate `other`'s particles after these (body.py:641-645); an
        attribute present on one side only is zero-filled on the other."""
        if not other.n:
            return
        mine, theirs = self._arrays(), other._arrays()
        for k in set(mine) | set(theirs):
            a, b = mine.get(k), theirs.get(k)
            if a is None:
                a = torch.zeros(self.n, dtype=b.dtype, device=b.device)
            if b is None:
                b = torch.zeros(other.n, dtype=a.dtype, device=a.device)
            setattr(self, k, torch.cat((a, b)))
        self.n += other.n

    def __getitem__(self, slc):
        new = ParticleSystem.__new__(ParticleSystem)
        new.__dict__["_device"] = self._device
        for k, v in self._arrays().items():
            setattr(new, k, v[slc].contiguous())
        new.n = int(new.mass.shape[0])
        return new

    def __len__(self):
        return self.n

    def to_numpy(self):
        return {k: v.detach().cpu().numpy() for k, v in self._arrays().items()}

    # ---- gravity (body.py:324-361) ---------------------------------------------
    def set_tstep(self, ps, eta):
        extensions.tstep.calc(self, ps, eta)

    def set_phi(self, ps):
        extensions.phi.calc(self, ps)

    def set_acc(self, ps):
        extensions.acc.calc(self, ps)

    def set_pnacc(self, ps):
        extensions.pnacc.calc(self, ps)

    def set_acc_jerk(self, ps):
        extensions.acc_jerk.calc(self, ps)

    def set_snap_crackle(self, ps):
        extensions.snap_crackle.calc(self, ps)

    def min_tstep(self):
        return float(self.tstep.abs().min())

    def max_tstep(self):
        return float(self.tstep.abs().max())

    # ---- diagnostics (body.py:74-321), reduced on the GPU in FP64 ------------
    # Sums go through tg_sum (numpy's pairwise order), so each value equals
    # the reference's numpy reduction of the same arrays bit for bit.
    @property
    def total_mass(self):
        return psum(self.mass)

    @property
    def com_r(self):
        m = self.mass
        return np.array([psum(m * self.rx), psum(m * self.ry), psum(m * self.rz)]) / self.total_mass

    @property
    def com_v(self):
        m = self.mass
        return np.array([psum(m * self.vx), psum(m * self.vy), psum(m * self.vz)]) / self.total_mass

    def com_move_to(self, com_r, com_v):
        self.rx += float(com_r[0]); self.ry += float(com_r[1]); self.rz += float(com_r[2])
        self.vx += float(com_v[0]); self.vy += float(com_v[1]); self.vz += float(com_v[2])

    def com_to_origin(self):
        self.com_move_to(-self.com_r, -self.com_v)

    @property
    def linear_momentum(self):
        m = self.mass
        return torch.stack([(m * self.vx).sum(), (m * self.vy).sum(), (m * self.vz).sum()]).cpu().numpy()

    @property
    def angular_momentum(self):
        m = self.mass
        px, py, pz = m * self.vx, m * self.vy, m * self.vz
        return torch.stack([(self.ry * pz - self.rz * py).sum(),
                            (self.rz * px - self.rx * pz).sum(),
                            (self.rx * py - self.ry * px).sum()]).cpu().numpy()

    @property
    def ke(self):
        return 0.5 * self.mass * (self.vx ** 2 + self.vy ** 2 + self.vz ** 2)

    @property
    def kinetic_energy(self):
        return psum(self.ke)

    @property
    def pe(self):
        self.set_phi(self)
        return self.mass * self.phi

    @property
    def potential_energy(self):
        return 0.5 * psum(self.pe)

    @property
    def virial_energy(self):
        return 2 * self.kinetic_energy + self.potential_energy

    @property
    def virial_radius(self):
        return (self.total_mass ** 2) / (-2 * self.potential_energy)

    def dynrescale_total_mass(self, total_mass):
        ratio = total_mass / self.total_mass
        self.mass *= ratio
        self.rx *= ratio; self.ry *= ratio; self.rz *= ratio

    def dynrescale_radial_size(self, size):
        com = self.com_r
        I = float((self.mass * ((self.rx - com[0]) ** 2 + (self.ry - com[1]) ** 2 + (self.rz - com[2]) ** 2)).sum())
        ratio = size / (I / self.total_mass) ** 0.5
        v_ratio = 1 / ratio ** 0.5
        self.rx *= ratio; self.ry *= ratio; self.rz *= ratio
        self.vx *= v_ratio; self.vy *= v_ratio; self.vz *= v_ratio

    def dynrescale_virial_radius(self, rvir):
        ratio = rvir / self.virial_radius
        v_ratio = 1 / ratio ** 0.5
        self.rx *= ratio; self.ry *= ratio; self.rz *= ratio
        self.vx *= v_ratio; self.vy *= v_ratio; self.vz *= v_ratio

    def scale_to_virial(self):
        ke = self.kinetic_energy
        pe = self.potential_energy
        ratio = (-0.5 * pe / ke) ** 0.5
        self.vx *= ratio; self.vy *= ratio; self.vz *= ratio

    def to_nbody_units(self):
        self.dynrescale_total_mass(1.0)
        ke, pe = self.kinetic_energy, self.potential_energy
        self.dynrescale_virial_radius(1.0)
        self.scale_to_virial()
