"""Initial conditions: Plummer spheres, a Salpeter mass function and binaries.

Restates the generators of tupan/ics/plummer.py:21-221 (Plummer.set_pos:
mass-stratified radii r = (m^(-2/3) - 1)^(-1/2) with mfrac = 0.999;
set_vel: |v| = sqrt(-2 q phi) with q drawn from the triangular density
2(1 - q) by pairwise rejection; per-particle eps2 = eps^2 / 2 for constant
softening; then com_to_origin, to_nbody_units and scale_to_virial) and, as
tupan/ics/fewbody.py:13-50 does, a two-body orbit of given a, e (here
starting at pericentre).  The potential
used by make_plummer for the velocities and the unit scalings comes from the
GPU Phi kernel; plummer_arrays needs no GPU and imports nothing of the
compiled library (the CPU baseline builds its workload with it).
Random numbers come from numpy.random.Generator(PCG64(seed)).

The Salpeter IMF draws dN/dm ~ m^-2.35 on [mlow, mhigh] by inverse CDF; the
reference's IMF class refuses mlow < 0.4 (ics/imf.py:85-88), so this one is
used for the [0.1, 100] range of the precision workload.

`IMF` has the reference's mass functions (ics/imf.py:67-112: equal mass,
Salpeter 1955, Padoan et al. 2007, Parravano et al. 2011), each normalised
over its own mass range and sampled by rejection under its peak from a
log-uniform proposal; drawn from numpy's global random state (rng=None)
they give the reference's samples for the same seed.
"""
import numpy as np


class Salpeter(object):
    def __init__(self, mlow=0.1, mhigh=100.0, alpha=-2.35):
        self.mlow, self.mhigh, self.alpha = float(mlow), float(mhigh), float(alpha)

    def sample(self, n, rng):
        a = self.alpha + 1.0
        u = rng.random(n)
        lo, hi = self.mlow ** a, self.mhigh ** a
        return (lo + u * (hi - lo)) ** (1.0 / a)


class EqualMass(object):
    def sample(self, n, rng):
        return np.ones(n)


class IMFSample(object):
    """A mass function f(m) restricted to [mlow, mhigh] inside the range
    [min_mlow, max_mhigh] it is defined on (tupan/ics/imf.py:20-64): f is
    normalised by the integral of f(m)/m over the whole range, its peak is
    located on that range, and a sample keeps the log-uniform proposals m
    with u * peak < f(m), u uniform, from batches that grow until one
    batch holds n accepted masses."""

    def __init__(self, func, min_mlow, max_mhigh, mlow, mhigh):
        from scipy.integrate import quad
        from scipy.optimize import fminbound
        if mlow < min_mlow or mhigh > max_mhigh:
            raise ValueError("Mass range outer of limits [{0}:{1}].".format(min_mlow, max_mhigh))
        norm = quad(lambda m: func(m) / m, min_mlow, max_mhigh)[0]
        self.func = lambda m: func(m) / norm
        self.mpeak = float(fminbound(lambda m: -self.func(m), min_mlow, max_mhigh, xtol=1.0e-8))
        self.peak = self.func(self.mpeak)
        self.mlow, self.mhigh = mlow, mhigh
        self.min_mlow, self.max_mhigh = min_mlow, max_mhigh

    def sample(self, n, rng=None):
        r = np.random if rng is None else rng
        size, kept = n, np.empty(0)
        while len(kept) < n:
            u = r.uniform(0.0, self.peak, size=size)
            m = np.exp(r.uniform(np.log(self.mlow), np.log(self.mhigh), size=size))
            kept = m[u < self.func(m)]
            size *= int(1 + n / max(len(kept), 1))
        return kept[:n]


class IMF(object):
    """The reference's mass functions (tupan/ics/imf.py:67-112)."""

    @staticmethod
    def equalmass():
        return IMFSample(lambda m: (1.0 + m) - m, 0.1, 10.0, 1.0, 1.0)

    @staticmethod
    def salpeter1955(mlow, mhigh):
        return IMFSample(lambda m: m ** (-1.35), 0.4, 120.0, mlow, mhigh)

    @staticmethod
    def padoan2007(mlow, mhigh):
        from scipy.special import erf
        gamma, m_ch, sigma = 1.4, 1.0, 1.8
        return IMFSample(lambda m: (m ** (-gamma)) * (1.0 + erf((4.0 * np.log(m / m_ch) + sigma ** 2)
                                                              / (np.sqrt(8.0) * sigma))),
                         0.004, 120.0, mlow, mhigh)

    @staticmethod
    def parravano2011(mlow, mhigh):
        return IMFSample(lambda m: (m ** (-1.35)) * (1.0 - np.exp(-(m / 0.35) ** (0.51 + 1.35))),
                         0.004, 120.0, mlow, mhigh)


def plummer_positions(n, rng, mfrac=0.999):
    irand = rng.permutation(n)
    mrand = (irand + rng.random(n)) * mfrac / n
    radius = 1.0 / np.sqrt(np.power(mrand, -2.0 / 3.0) - 1.0)
    theta = np.arccos(rng.uniform(-1.0, 1.0, size=n))
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    return (radius * np.sin(theta) * np.cos(phi), radius * np.sin(theta) * np.sin(phi),
            radius * np.cos(theta))


def triangular(n, rng):
    """q with density 2(1 - q) on [0, 1]: keep r2 when r2 < r1."""
    out = np.empty(0)
    while out.size < n:
        r1 = rng.random(2 * n)
        r2 = rng.random(2 * n)
        out = np.concatenate([out, r2[r2 < r1]])
    return out[:n]


def _gpu_phi(mass, rx, ry, rz, eps2, device=None):
    """phi_i = -sum_j m_j / sqrt(r_ij^2 + e2_i + e2_j) by the FP64 kernel
    (bit-identical to the reference C backend)."""
    from .lib import extensions
    from .particles import ParticleSystem
    ps = ParticleSystem.from_arrays(device=device, mass=mass, rx=rx, ry=ry, rz=rz, eps2=eps2)
    extensions.Phi("CUDA", "float64").calc(ps, ps)
    return ps.phi.cpu().numpy()


def plummer_reference(n, eps, imf, seed=None, mfrac=0.999, softening_type=0, device=None, phi=None):
    """The reference's Plummer model, value for value (tupan/ics/plummer.py:
    22-133, 213-221): masses from the mass function `imf` (a tuple such as
    ("equalmass",) or ("salpeter1955", 0.5, 100.0) naming an `IMF`, or any
    object with .sample(n)), softening of `softening_type` 0-4 scaled to a
    mean of eps^2 and halved, positions from the random state the masses
    started from, speeds sqrt(-2 q phi) with q drawn pair by pair, then the
    centre of mass moved to the origin, N-body units and virial
    equilibrium, each step with the reference's numpy expressions, all
    drawn from numpy's global random state seeded with `seed`.  The
    potential comes from `phi(mass, rx, ry, rz, eps2)`, by default the FP64
    Phi kernel on the GPU, which the reference computes with its C backend
    to the same bits; so for the same seed the particle set equals the
    reference's make_plummer.  Returns a ParticleSystem on `device`."""
    from .particles import ParticleSystem
    n = max(int(n), 2)
    if isinstance(imf, (tuple, list)):
        imf = getattr(IMF, imf[0])(*imf[1:])
    if phi is None:
        def phi(*a):
            return _gpu_phi(*a, device=device)
    np.random.seed(seed)
    ilist = np.arange(n)
    srand = np.random.get_state()
    mass = np.zeros(n)
    mass[...] = imf.sample(n)
    mass /= float(mass.sum())
    if softening_type == 0:
        e2 = np.ones(n)
    elif softening_type == 1:
        e2 = mass ** 2
    elif softening_type == 2:
        e2 = mass / n
    elif softening_type == 3:
        e2 = (mass / n ** 2) ** (2.0 / 3)
    elif softening_type == 4:
        e2 = (1.0 / (mass * n ** 2)) ** 2
    else:
        raise ValueError("Unexpected value for softening_type: {}.".format(softening_type))
    e2 *= (eps * eps) / np.mean(e2)
    eps2 = e2 / 2
    np.random.set_state(srand)
    irand = np.random.permutation(ilist)
    mrand = (irand + np.random.random(n)) * mfrac / n
    radius = 1.0 / np.sqrt(np.power(mrand, -2.0 / 3.0) - 1.0)
    theta = np.arccos(np.random.uniform(-1.0, 1.0, size=n))
    ang = np.random.uniform(0.0, 2.0 * np.pi, size=n)
    rx = radius * np.sin(theta) * np.cos(ang)
    ry = radius * np.sin(theta) * np.sin(ang)
    rz = radius * np.cos(theta)
    pot = phi(mass, rx, ry, rz, eps2)
    rnd = np.empty(n)
    count = 0
    while count < n:                     # q with density 2(1 - q), one pair at a time
        r1 = np.random.random()
        r2 = np.random.random()
        if r2 < r1:
            rnd[count] = r2
            count += 1
    speed = np.sqrt(-2 * rnd * pot)
    theta = np.arccos(np.random.uniform(-1.0, 1.0, size=n))
    ang = np.random.uniform(0.0, 2.0 * np.pi, size=n)
    vx = speed * np.sin(theta) * np.cos(ang)
    vy = speed * np.sin(theta) * np.sin(ang)
    vz = speed * np.cos(theta)

    def total_mass():
        return float(mass.sum())

    def potential_energy():
        return 0.5 * float((mass * phi(mass, rx, ry, rz, eps2)).sum())

    # com_to_origin (body.py:85-176)
    mtot = total_mass()
    com_r = np.array([mass * rx, mass * ry, mass * rz]).T.sum(0) / mtot
    com_v = np.array([mass * vx, mass * vy, mass * vz]).T.sum(0) / mtot
    for a, c in ((rx, -com_r[0]), (ry, -com_r[1]), (rz, -com_r[2]),
                 (vx, -com_v[0]), (vy, -com_v[1]), (vz, -com_v[2])):
        a += c
    # to_nbody_units: dynrescale_total_mass(1.0), dynrescale_virial_radius(1.0) (body.py:405-461)
    m_ratio = 1.0 / total_mass()
    for a in (mass, rx, ry, rz):
        a *= m_ratio
    r_scale = 1.0 / (total_mass() ** 2 / (-2 * potential_energy()))
    v_scale = 1 / r_scale ** 0.5
    for a in (rx, ry, rz):
        a *= r_scale
    for a in (vx, vy, vz):
        a *= v_scale
    # scale_to_virial (body.py:444-453)
    ke = float((0.5 * mass * (vx ** 2 + vy ** 2 + vz ** 2)).sum())
    pe = potential_energy()
    v_scale = ((-0.5 * pe) / ke) ** 0.5
    for a in (vx, vy, vz):
        a *= v_scale
    return ParticleSystem.from_arrays(device=device, id=ilist, mass=mass, eps2=eps2, rx=rx, ry=ry, rz=rz,
                                      vx=vx, vy=vy, vz=vz)


def make_plummer(n, eps, imf=None, seed=0, device=None, prec="float64"):
    """Plummer sphere in N-body (Henon) units: M = 1, E = -1/4, Q = 1/2.
    With `imf` given as the reference's tuple (("equalmass",),
    ("salpeter1955", mlow, mhigh), ...) this is plummer_reference: the
    reference's own model for that seed."""
    if isinstance(imf, (tuple, list)):
        return plummer_reference(n, eps, imf, seed=seed, device=device)
    from .lib import extensions
    from .particles import ParticleSystem
    rng = np.random.default_rng(seed)
    imf = imf or EqualMass()
    mass = imf.sample(n, rng)
    mass = mass / mass.sum()
    ps = ParticleSystem(n, device=device)
    ps.set_array("mass", mass)
    ps.set_array("eps2", np.full(n, eps * eps / 2.0))
    rx, ry, rz = plummer_positions(n, rng)
    ps.set_array("rx", rx); ps.set_array("ry", ry); ps.set_array("rz", rz)
    extensions.Phi("CUDA", prec).calc(ps, ps)
    q = triangular(n, rng)
    v = np.sqrt(-2.0 * q * ps.phi.cpu().numpy())
    theta = np.arccos(rng.uniform(-1.0, 1.0, size=n))
    phi = rng.uniform(0.0, 2.0 * np.pi, size=n)
    ps.set_array("vx", v * np.sin(theta) * np.cos(phi))
    ps.set_array("vy", v * np.sin(theta) * np.sin(phi))
    ps.set_array("vz", v * np.cos(theta))
    ps.com_to_origin()
    ps.to_nbody_units()
    ps.scale_to_virial()
    return ps


def make_binary(m1, m2, a, e, rng=None):
    """Two bodies on a Kepler orbit of semi-major axis a and eccentricity e,
    centre of mass at rest, optionally in a random orientation.  The
    relative orbit starts at pericentre; the reference's make_binary
    (tupan/ics/fewbody.py:13-50) starts it at apocentre, along x with the
    velocities along y."""
    m = m1 + m2
    rp = a * (1 - e)
    vp = np.sqrt(m * (1 + e) / rp)
    r = np.array([[m2 / m * rp, 0, 0], [-m1 / m * rp, 0, 0]])
    v = np.array([[0, m2 / m * vp, 0], [0, -m1 / m * vp, 0]])
    if rng is not None:   # random orientation
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        r, v = r @ q.T, v @ q.T
    return np.array([m1, m2]), r, v


def plummer_arrays(n, eps, imf=None, seed=0, mfrac=0.999):
    """Host-only Plummer sphere (numpy arrays) for benchmarks and CPU tests.

    Same sampling as make_plummer, but the potential used for the velocity
    magnitudes is the smooth Plummer potential -1/sqrt(1 + r^2), the
    scaling to Henon units is the analytic one (length 3 pi / 16, velocity
    its inverse square root), and the speeds are then scaled so that the
    kinetic energy is the model's 1/4 (virial ratio 1/2 against its
    potential energy -1/2, the role of make_plummer's scale_to_virial), so
    no O(N^2) pass is needed.
    """
    rng = np.random.default_rng(seed)
    imf = imf or EqualMass()
    mass = imf.sample(n, rng)
    mass = mass / mass.sum()
    rx, ry, rz = plummer_positions(n, rng, mfrac)
    pot = -1.0 / np.sqrt(1.0 + rx * rx + ry * ry + rz * rz)
    q = triangular(n, rng)
    v = np.sqrt(-2.0 * q * pot)
    theta = np.arccos(rng.uniform(-1.0, 1.0, size=n))
    ph = rng.uniform(0.0, 2.0 * np.pi, size=n)
    vx, vy, vz = v * np.sin(theta) * np.cos(ph), v * np.sin(theta) * np.sin(ph), v * np.cos(theta)
    s = 3.0 * np.pi / 16.0
    d = {"mass": mass, "eps2": np.full(n, eps * eps / 2.0)}
    for k, (r, u) in zip("xyz", ((rx, vx), (ry, vy), (rz, vz))):
        d["r" + k] = (r - np.dot(mass, r)) * s
        d["v" + k] = (u - np.dot(mass, u)) / np.sqrt(s)
    ke = 0.5 * np.dot(mass, d["vx"] ** 2 + d["vy"] ** 2 + d["vz"] ** 2)
    if ke > 0:
        f = np.sqrt(0.25 / ke)
        for k in "xyz":
            d["v" + k] = d["v" + k] * f
    return d
