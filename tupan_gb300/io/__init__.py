"""Snapshot and worldline files (tupan/io/__init__.py:13-113, hdf5io.py:23-146).

    io = IO("run.hdf5", "a")
    io.dump_snapshot(ps, snap_number=3)     # /Snapshot_000003/particlesystem/bodies
    io.dump_worldline(wl)                   # rows appended to /Worldline/particlesystem/bodies
    ps = IO("run.hdf5", "r").load_snapshot(3)

The file layout is the reference's, so files move between the two in both
directions: a group per snapshot ("Snapshot", or "Snapshot_%06d" for a
numbered one), inside it a group named after the particle-system class with
a "Class" attribute, and one dataset per particle kind ("bodies" here) of
compound records with the Bodies fields of tupan/particles/body.py:26-39 (id
and nstep unsigned 64-bit, the rest float64), chunked, of unlimited extent,
shuffle+deflate compressed, with its own "Class" attribute.  Dumping into an
existing snapshot or worldline appends rows, as the reference's
`store_dset` does.  The Class attributes hold the protocol-0 pickle text of
the reference's classes (what h5py stores there); reading parses the class
name from that text and never unpickles it.  A particle set of the
reference's own classes (its numpy ParticleSystem, handed to this IO as the
dumpper of its integrators) is stored as the reference stores it: one
dataset per particle kind ("bodies", "stars", "blackholes", "sphs") of that
kind's `get_state()` records, each with its own class.

The particles live on the GPU: a dump gathers the record fields of the set on
the device, copies them into pinned host memory in one asynchronous transfer
per block (float64 and int64 rows) and encodes them on the host, deflating
the chunks on a thread pool.  With `background=True` the encoding,
compression and file writes run on a writer thread, so an integrator that dumps its worldline
every step does not wait for zlib; `flush()` (called by every load, by
`close()` and at interpreter exit) waits for the queued writes and re-raises
the first error of the writer; a load also waits for the writes other IO
objects have queued for the same file.

A ".psdf" name selects a PSDF stream (tupan_gb300.io.psdf): one YAML
`!Particle` document per particle with the keys of psdfio.py's
`Stream.to_yaml` (position, velocity, mass, id, time, softening, and the
acceleration and potential when the set carries them); dumps append to the
stream, a load reads every particle in it, and `to_psdf` / `to_hdf5`
convert between the two formats as hdf5io.py:134-146 and psdfio.py:46-57 do.

Differences from the reference: the reference's PSDF path cannot run as it
stands (tupan/io/__init__.py:28 constructs PSDFIO with two arguments,
psdfio.py:22 takes one; PSDFIO has neither dump_snapshot nor
dump_worldline); here it follows the mapping `Stream.to_yaml` and
`Stream.from_loader` define.  `load_worldline` returns the worldline's rows
(the reference's raises NotImplementedError, hdf5io.py:117-121).  A set
with several particle kinds loads as one set, the kinds' datasets in name
order, fields a kind lacks set to zero.
"""
import atexit
import logging
import os
import queue
import sys
import threading
import warnings

import numpy as np
import torch

from . import hdf5, psdf

__all__ = ["IO", "BODIES_FIELDS"]

# tupan/particles/body.py:26-39, in that order (uint = u8, real = f8)
BODIES_FIELDS = (("id", "<u8"), ("mass", "<f8"), ("eps2", "<f8"), ("rx", "<f8"), ("ry", "<f8"),
                 ("rz", "<f8"), ("vx", "<f8"), ("vy", "<f8"), ("vz", "<f8"), ("time", "<f8"),
                 ("nstep", "<u8"), ("tstep", "<f8"))
BODIES_DTYPE = np.dtype(list(BODIES_FIELDS))

GROUP_NAME = "particlesystem"          # type(ps).__name__.lower() in hdf5io.py:57
MEMBER_NAME = "bodies"                 # the members key of Bodies (allparticles.py:34)
SYSTEM_CLASS = ("tupan.particles.allparticles", "ParticleSystem")
MEMBER_CLASSES = {"bodies": ("tupan.particles.body", "Bodies"), "stars": ("tupan.particles.star", "Stars"),
                  "blackholes": ("tupan.particles.blackhole", "Blackholes"),
                  "sphs": ("tupan.particles.sph", "Sphs")}

logger = logging.getLogger(__name__)


def pickled_class(module, name):
    """The protocol-0 pickle text of a class reference, as hdf5io.py:42-43
    stores it: a GLOBAL opcode, a memo put and STOP."""
    return "c%s\n%s\np0\n." % (module, name)


def class_of(text):
    """(module, name) from a protocol-0 class pickle, without unpickling."""
    if not isinstance(text, str) or not text.startswith("c"):
        return None
    parts = text[1:].split("\n")
    return (parts[0], parts[1]) if len(parts) >= 2 else None


def snapshot_name(snap_number):
    """hdf5io.py:55-57"""
    return "Snapshot" + ("_" + str(snap_number).zfill(6) if isinstance(snap_number, int) else "")


# ---- device <-> records ----------------------------------------------------------------

class _Staged(object):
    """One dump in flight: host copies of the named attributes of a set and
    the event after which they are valid.  A tupan_gb300 ParticleSystem is
    gathered on the device (one index_select per block) and copied into
    pinned host buffers asynchronously; any other set (the reference's numpy
    ParticleSystem, given to this IO as the dumpper of the reference's own
    integrators) is read attribute by attribute."""

    def __init__(self, ps, names):
        self.names = list(names)
        self.cols = None
        self.event = None
        if not hasattr(ps, "_layout"):
            n = int(getattr(ps, "n", 0) or 0)
            self.cols = {}
            for k in self.names:      # copies: the set may change before a queued dump runs
                v = getattr(ps, k) if n else np.zeros(0)
                self.cols[k] = v.detach().cpu().numpy().copy() if isinstance(v, torch.Tensor) else np.array(v)
            return
        lay = ps._layout
        self.rnames = [k for k in self.names if lay[k][0] == "_real"]
        self.inames = [k for k in self.names if lay[k][0] == "_int"]
        dev = ps._real.device
        real = ps._real.index_select(0, torch.tensor([lay[k][1] for k in self.rnames], device=dev,
                                                     dtype=torch.int64))
        int_ = ps._int.index_select(0, torch.tensor([lay[k][1] for k in self.inames], device=dev,
                                                    dtype=torch.int64))
        if dev.type == "cuda":
            # pinned host buffers: on the Grace host a process's first copy
            # into pageable memory took 4 s, into pinned memory 0.1 s
            self.real = torch.empty(real.shape, dtype=real.dtype, pin_memory=True)
            self.int_ = torch.empty(int_.shape, dtype=int_.dtype, pin_memory=True)
            self.real.copy_(real, non_blocking=True)
            self.int_.copy_(int_, non_blocking=True)
            self.event = torch.cuda.Event()
            self.event.record()
        else:
            self.real, self.int_ = real.cpu(), int_.cpu()

    def columns(self):
        """name -> host numpy array"""
        if self.cols is None:
            if self.event is not None:
                self.event.synchronize()
            real, int_ = self.real.numpy(), self.int_.numpy()
            self.cols = {k: real[i] for i, k in enumerate(self.rnames)}
            self.cols.update({k: int_[i] for i, k in enumerate(self.inames)})
        return self.cols

    def records(self):
        """The Bodies records (BODIES_DTYPE) of the staged columns."""
        cols = self.columns()
        n = len(cols["id"])
        out = np.empty(n, dtype=BODIES_DTYPE)
        for k, t in BODIES_FIELDS:
            out[k] = cols[k].astype(np.uint64) if t == "<u8" else cols[k]
        return out


def particles_from_columns(cols, device=None):
    """A ParticleSystem from name -> 1-D numpy arrays: the Bodies fields and
    any other numeric field as an auxiliary attribute."""
    from ..particles import ParticleSystem
    n = len(cols["id"]) if "id" in cols else len(next(iter(cols.values())))
    ps = ParticleSystem(n, device=device)
    for k, v in cols.items():
        v = np.asarray(v)
        if v.dtype.kind in "iu":
            ps.set_array(k, torch.from_numpy(v.astype(np.int64)))
        elif v.dtype.kind == "f":
            ps.set_array(k, torch.from_numpy(v.astype(np.float64)))
    return ps


def particles_from_records(arrays, device=None):
    """A ParticleSystem from record arrays (one per particle kind), the kinds
    concatenated; a field a kind lacks is zero for its particles."""
    arrays = [a for a in arrays if len(a)]
    names = []
    for a in arrays:
        names += [k for k in a.dtype.names if k not in names]
    cols = {}
    for k in names:
        parts = []
        for a in arrays:
            if k in a.dtype.names:
                parts.append(np.asarray(a[k]).reshape(len(a), -1)[:, 0] if a[k].ndim > 1 else np.asarray(a[k]))
            else:
                parts.append(np.zeros(len(a)))
        cols[k] = np.concatenate(parts)
    if not cols:
        cols = {k: np.zeros(0, dtype=np.dtype(t)) for k, t in BODIES_FIELDS}
    return particles_from_columns(cols, device)


# ---- the writer thread -----------------------------------------------------------------

class _Writer(threading.Thread):
    def __init__(self):
        threading.Thread.__init__(self, name="tupan-io-writer", daemon=True)
        self.q = queue.Queue(maxsize=8)
        self.error = None
        self.start()

    def run(self):
        while True:
            job = self.q.get()
            try:
                if job is not None and self.error is None:
                    job()
            except BaseException as exc:          # kept for the caller's next flush
                self.error = exc
            finally:
                self.q.task_done()
            if job is None:
                return

    def submit(self, job):
        self.q.put(job)

    def flush(self):
        self.q.join()
        if self.error is not None:
            err, self.error = self.error, None
            raise err


_writers = []


@atexit.register
def _flush_all():
    for w in _writers:
        try:
            w.flush()
        except BaseException as exc:
            logger.error("snapshot writer: %s", exc)


# ---- the public interface --------------------------------------------------------------

class IO(object):
    """tupan/io/__init__.py:13-113: the file's extension picks the format."""
    PROVIDED_FORMATS = ["hdf5", "psdf"]

    def __init__(self, fname, fmode, background=False):
        self.fname = fname
        self.fmode = fmode
        self.background = background
        self._writer = None

    # -- helpers
    def _format(self):
        fname = self.fname
        if fname.endswith(".hdf5"):
            return "hdf5"
        if fname.endswith(".psdf"):
            return "psdf"
        raise NotImplementedError("Unknown format: '{}'. Choose from: {}".format(
            fname.rpartition('.')[-1], self.PROVIDED_FORMATS))

    def _submit(self, job):
        if not self.background:
            job()
            return
        if self._writer is None:
            self._writer = _Writer()
            self._writer.path = os.path.abspath(self.fname)
            _writers.append(self._writer)
        self._writer.submit(job)

    def flush(self):
        """Wait for the queued dumps; re-raise the writer's first error."""
        if self._writer is not None:
            self._writer.flush()

    def close(self):
        self.flush()
        if self._writer is not None:
            self._writer.submit(None)
            self._writer.join()
            _writers.remove(self._writer)
            self._writer = None

    def _dump(self, base, ps):
        fmt = self._format()
        fname, fmode = self.fname, self.fmode
        if fmt == "psdf":
            lay = getattr(ps, "_layout", None)
            extra = [k for k in psdf.VECTORS["a"] + ("phi",)
                     if (k in lay if lay is not None else hasattr(ps, k))]
            if len([k for k in extra if k != "phi"]) != 3:
                extra = [k for k in extra if k == "phi"]
            staged = _Staged(ps, [k for k, _t in BODIES_FIELDS] + extra)

            def job():
                text = psdf.dump_text(staged.columns())
                with open(fname, "w" if fmode == "w" else "a") as fobj:
                    fobj.write(text)
        elif not hasattr(ps, "_layout") and isinstance(getattr(ps, "members", None), dict):
            # the reference's ParticleSystem: one dataset per particle kind
            # with that kind's own records, as hdf5io.py:51-66 stores them
            group = type(ps).__name__.lower()
            gcls = pickled_class(type(ps).__module__, type(ps).__name__)
            kinds = [(key, pickled_class(type(obj).__module__, type(obj).__name__), obj.get_state())
                     for key, obj in sorted(ps.members.items()) if obj.n]

            def job():
                with hdf5.File(fname, fmode) as f:
                    g = f.require_group(base + "/" + group)
                    g.set_attr("Class", gcls)
                    for key, cls, rows in kinds:
                        g.append_rows(key, rows).set_attr("Class", cls)
        else:
            staged = _Staged(ps, [k for k, _t in BODIES_FIELDS])

            def job():
                rows = staged.records()
                with hdf5.File(fname, fmode) as f:
                    g = f.require_group(base + "/" + GROUP_NAME)
                    g.set_attr("Class", pickled_class(*SYSTEM_CLASS))
                    if len(rows):
                        ds = g.append_rows(MEMBER_NAME, rows)
                        ds.set_attr("Class", pickled_class(*MEMBER_CLASSES[MEMBER_NAME]))
        self._submit(job)

    def _load(self, base, device):
        self.flush()
        path = os.path.abspath(self.fname)
        for w in list(_writers):            # dumps other IO objects queued for this file
            if w.path == path:
                w.flush()
        if not os.path.exists(self.fname):
            warnings.warn("No such file or directory: '{}'".format(self.fname), stacklevel=3)
            sys.exit()
        try:
            if self._format() == "psdf":
                with open(self.fname) as fobj:
                    return particles_from_columns(psdf.columns_from_docs(psdf.parse_text(fobj.read())),
                                                  device)
            with hdf5.File(self.fname, "r") as f:
                top = f[base]
                groups = top.values()
                if not groups:
                    raise ValueError("group %s is empty" % base)
                group = groups[0]                   # hdf5io.py:81
                arrays = [ds.read() for ds in group.values() if isinstance(ds, hdf5.Dataset)]
        except NotImplementedError:
            raise
        except Exception as exc:
            logger.exception(str(exc))
            raise ValueError("File not in a supported format.")
        return particles_from_records(arrays, device)

    # -- tupan/io/__init__.py:22-113
    def dump_snapshot(self, ps, snap_number=None):
        """hdf5io.py:51-72; a PSDF stream has no snapshot groups: the
        particles are appended to it."""
        self._dump(snapshot_name(snap_number), ps)

    def load_snapshot(self, snap_number=None, device=None):
        """hdf5io.py:74-95; for a PSDF stream, every particle in it."""
        return self._load(snapshot_name(snap_number), device)

    def dump_worldline(self, wl):
        """hdf5io.py:97-115"""
        self._dump("Worldline", wl)

    def load_worldline(self, wl_number=None, device=None):
        """Every row the worldline dumps appended, in the order they were
        written."""
        return self._load("Worldline", device)

    def to_psdf(self):
        """An HDF5 file's snapshot (or, without one, its worldline) as a PSDF
        stream beside it (hdf5io.py:134-146)."""
        if self._format() != "hdf5":
            raise ValueError("This file is already in 'psdf' format!")
        try:
            ps = self.load_snapshot(device="cpu")
        except ValueError:
            ps = self.load_worldline(device="cpu")
        IO(self.fname[:-len(".hdf5")] + ".psdf", "w").dump_snapshot(ps)

    def to_hdf5(self):
        """A PSDF stream as the snapshot of an HDF5 file beside it
        (psdfio.py:46-57)."""
        if self._format() != "psdf":
            raise ValueError("This file is already in 'hdf5' format!")
        ps = self.load_snapshot(device="cpu")
        IO(self.fname[:-len(".psdf")] + ".hdf5", "w").dump_snapshot(ps)
