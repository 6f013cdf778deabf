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


SPARE_ROWS = 24   # room for kernel outputs registered later, without reallocation


def _layout(rnames, inames):
    """attribute name -> (block, row)"""
    lay = {k: ("_real", r) for r, k in enumerate(rnames)}
    lay.update({k: ("_int", r) for r, k in enumerate(inames)})
    return lay


class ParticleSystem(object):
    """n particles; every attribute is a length-n tensor on `device`.

    Storage: all float64 attributes are the rows of one 2-D tensor and the
    int64 ones (id, nstep) of another, each with spare rows for attributes
    registered later; an attribute is a contiguous row view.  Selecting,
    copying or concatenating particles is then one gather or one cat per
    block instead of one per attribute, which is what keeps the
    hierarchical integrators' many small subsets cheap.  Assigning a tensor
    to an attribute copies it into the attribute's row."""

    include_pn_corrections = False
    t_curr = 0.0

    def __init__(self, n=0, device=None, **arrays):
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
        d = self.__dict__
        d["_device"] = torch.device(device)
        d["n"] = int(n)
        d["_rnames"] = list(REAL_ATTRS)
        d["_inames"] = list(INT_ATTRS)
        d["_real"] = torch.zeros(len(REAL_ATTRS) + SPARE_ROWS, d["n"], dtype=torch.float64, device=d["_device"])
        d["_int"] = torch.zeros(len(INT_ATTRS) + 2, d["n"], dtype=torch.int64, device=d["_device"])
        d["_int"][INT_ATTRS.index("id")] = torch.arange(d["n"], dtype=torch.int64, device=d["_device"])
        d["_layout"] = _layout(d["_rnames"], d["_inames"])
        for k, v in arrays.items():
            self.set_array(k, v)

    @classmethod
    def _from_blocks(cls, device, n, rnames, inames, real, int_, layout=None):
        # the name lists and the layout are shared with the source set: they
        # are replaced, never changed in place
        new = cls.__new__(cls)
        d = new.__dict__
        d["_device"] = device
        d["n"] = int(n)
        d["_rnames"] = rnames
        d["_inames"] = inames
        d["_real"] = real
        d["_int"] = int_
        d["_layout"] = layout if layout is not None else _layout(rnames, inames)
        return new

    def __getattr__(self, name):
        # only reached for names not in __dict__: an attribute's row view is
        # made on first use and cached
        d = self.__dict__
        lay = d.get("_layout")
        if lay is not None and name in lay:
            key, r = lay[name]
            v = d[key][r]
            d[name] = v
            return v
        raise AttributeError(name)

    def _rebind(self):
        # the blocks were replaced: drop the cached row views
        d = self.__dict__
        for k in d["_layout"]:
            d.pop(k, None)

    def _add_row(self, name, value):
        d = self.__dict__
        is_int = value.dtype in (torch.int64, torch.int32, torch.bool)
        nkey, key = ("_inames", "_int") if is_int else ("_rnames", "_real")
        names = d[nkey]
        blk = d[key]
        if len(names) == blk.shape[0]:   # no spare row left: grow the block
            grown = torch.zeros(blk.shape[0] + SPARE_ROWS, d["n"], dtype=blk.dtype, device=blk.device)
            grown[:blk.shape[0]] = blk
            self._rebind()
            d[key] = blk = grown
        blk[len(names)].copy_(value)
        d[nkey] = names + [name]
        d["_layout"] = _layout(d["_rnames"], d["_inames"])

    def __setattr__(self, name, value):
        d = self.__dict__
        if isinstance(value, torch.Tensor) and not name.startswith("_"):
            if value.dim() != 1 or value.shape[0] != d["n"]:
                raise ValueError("%s must have shape (%d,)" % (name, d["n"]))
            if name in d["_layout"]:
                row = getattr(self, name)
                if value.data_ptr() != row.data_ptr():
                    row.copy_(value)
            else:
                self._add_row(name, value)
            return
        d[name] = value

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
        if attr in self.__dict__ or attr in self.__dict__["_layout"]:
            raise ValueError("'{0}' is already a registered attribute.".format(attr))
        dtype = torch.float64 if sctype == "real" else torch.int64
        self._add_row(attr, torch.zeros(self.n, dtype=dtype, device=self._device))

    def _arrays(self):
        d = self.__dict__
        return {k: getattr(self, k) for k in d["_rnames"] + d["_inames"]}

    def copy(self):
        return ParticleSystem._from_blocks(self._device, self.n, self._rnames, self._inames,
                                           self._real.clone(), self._int.clone(), self._layout)

    def append(self, other):
        """Concatenate `other`'s particles after these (body.py:641-645); an
        attribute present on one side only is zero-filled on the other."""
        if not other.n:
            return
        d = self.__dict__
        if (other._rnames == d["_rnames"] and other._inames == d["_inames"]
                and other._real.shape[0] == d["_real"].shape[0] and other._int.shape[0] == d["_int"].shape[0]):
            self._rebind()
            d["_real"] = torch.cat((d["_real"], other._real), dim=1)
            d["_int"] = torch.cat((d["_int"], other._int), dim=1)
        else:
            mine, theirs = self._arrays(), other._arrays()
            rn = d["_rnames"] + [k for k in other._rnames if k not in d["_rnames"]]
            inn = d["_inames"] + [k for k in other._inames if k not in d["_inames"]]
            n = d["n"] + other.n
            real = torch.zeros(len(rn) + SPARE_ROWS, n, dtype=torch.float64, device=self._device)
            int_ = torch.zeros(len(inn) + 2, n, dtype=torch.int64, device=self._device)
            for blk, names in ((real, rn), (int_, inn)):
                for r, k in enumerate(names):
                    if k in mine:
                        blk[r, :d["n"]] = mine[k]
                    if k in theirs:
                        blk[r, d["n"]:] = theirs[k]
            self._rebind()
            d["_real"], d["_int"], d["_rnames"], d["_inames"] = real, int_, rn, inn
            d["_layout"] = _layout(rn, inn)
        d["n"] += other.n

    def __getitem__(self, slc):
        if isinstance(slc, torch.Tensor) and slc.dtype == torch.bool:
            # one index computation (one host sync) instead of one per attribute
            return self.take(torch.nonzero(slc).flatten())
        if isinstance(slc, torch.Tensor):
            return self.take(slc.to(device=self._device, dtype=torch.int64))
        real = self._real[:, slc].contiguous()
        int_ = self._int[:, slc].contiguous()
        return ParticleSystem._from_blocks(self._device, real.shape[1], self._rnames, self._inames, real, int_,
                                           self._layout)

    def take(self, idx):
        """The particles at device indices `idx`, in that order (one gather per
        block, no host synchronisation)."""
        return ParticleSystem._from_blocks(self._device, idx.numel(), self._rnames, self._inames,
                                           self._real.index_select(1, idx), self._int.index_select(1, idx),
                                           self._layout)

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
