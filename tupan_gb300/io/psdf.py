"""PSDF particle streams: YAML documents, one `!Particle` mapping per particle
(tupan/io/psdfio.py:60-218).

The reference writes them with PyYAML (`yaml.dump_all(..., default_flow_style
=False, explicit_start=True)` of `Stream.to_yaml` mappings) and reads them back
with `Stream.from_loader`.  Neither PyYAML nor any other YAML library is
available here, so this module emits the same text PyYAML emits for those
documents and parses the subset of YAML they use: documents opened by
`---` (with or without the `!Particle` tag), `key: scalar` lines, and
three-component vectors as block sequences (`- x` lines) or flow sequences
(`[x, y, z]`).

Keys, in the sorted order PyYAML writes them (psdfio.py:72-92, 161-175):

    a      acceleration [ax, ay, az]  (written when the set carries ax, ay, az)
    eps2   squared softening
    id     particle index
    m      mass
    pot    potential (written when the set carries phi)
    r      position [rx, ry, rz]
    t      the particle's time
    type   particle kind ("body"; "blackhole" and "sph" are read as bodies)
    v      velocity [vx, vy, vz]

Floats are written as PyYAML writes them (Python's shortest round-trip repr,
".0" added before an exponent without a decimal point, .inf / .nan), so a
stream read back gives the same float64 values.  The reference's stream
writer cannot run as it stands (psdfio.py:22 takes one constructor argument
where tupan/io/__init__.py:28 passes two, and `Stream.to_dumper` iterates a
particle API the particle classes no longer have); these streams follow the
mapping its `to_yaml` and `from_loader` define.
"""
import math

import numpy as np

VECTORS = {"r": ("rx", "ry", "rz"), "v": ("vx", "vy", "vz"), "a": ("ax", "ay", "az")}
SCALARS = {"eps2": "eps2", "id": "id", "m": "mass", "pot": "phi", "t": "time"}
KINDS = ("body", "blackhole", "sph")


def yaml_float(x):
    """PyYAML's representation of a float."""
    x = float(x)
    if x != x:
        return ".nan"
    if math.isinf(x):
        return ".inf" if x > 0 else "-.inf"
    s = repr(x).lower()
    if "." not in s and "e" in s:
        s = s.replace("e", ".0e", 1)
    return s


def _parse_scalar(s):
    s = s.strip()
    low = s.lower()
    if low == ".nan":
        return float("nan")
    if low in (".inf", "+.inf"):
        return float("inf")
    if low == "-.inf":
        return float("-inf")
    try:
        return int(s)
    except ValueError:
        pass
    try:
        return float(s)
    except ValueError:
        return s.strip("'\"")


def dump_text(columns):
    """Stream text for the particles in `columns` (name -> 1-D numpy array)."""
    n = len(columns["id"])
    has_a = all(k in columns for k in VECTORS["a"])
    has_pot = "phi" in columns
    out = []
    for i in range(n):
        doc = ["--- !Particle"]
        if has_a:
            doc.append("a:")
            doc += ["- " + yaml_float(columns[k][i]) for k in VECTORS["a"]]
        doc.append("eps2: " + yaml_float(columns["eps2"][i]))
        doc.append("id: %d" % int(columns["id"][i]))
        doc.append("m: " + yaml_float(columns["mass"][i]))
        if has_pot:
            doc.append("pot: " + yaml_float(columns["phi"][i]))
        doc.append("r:")
        doc += ["- " + yaml_float(columns[k][i]) for k in VECTORS["r"]]
        doc.append("t: " + yaml_float(columns["time"][i]))
        doc.append("type: body")
        doc.append("v:")
        doc += ["- " + yaml_float(columns[k][i]) for k in VECTORS["v"]]
        out.append("\n".join(doc))
    return "\n".join(out) + ("\n" if out else "")


def parse_text(text):
    """The documents of a stream as dicts (vectors as lists)."""
    docs, cur, key = [], None, None
    for raw in text.splitlines():
        line = raw.split(" #", 1)[0].rstrip()
        if (not line.strip() or line.lstrip().startswith("#") or line.startswith("%")
                or line.strip() == "..."):
            continue
        if line.startswith("---"):
            cur, key = {}, None
            docs.append(cur)
            rest = line[3:].strip()
            if rest and not rest.startswith("!"):
                raise ValueError("unexpected content after '---': %r" % rest)
            continue
        if cur is None:                      # a stream without a leading '---'
            cur = {}
            docs.append(cur)
        s = line.strip()
        if s.startswith("- "):
            if key is None or not isinstance(cur.get(key), list):
                raise ValueError("sequence item outside a sequence: %r" % raw)
            cur[key].append(_parse_scalar(s[2:]))
            continue
        if ":" not in s:
            raise ValueError("not a mapping entry: %r" % raw)
        k, v = s.split(":", 1)
        k, v = k.strip(), v.strip()
        if not v:
            cur[k] = []
            key = k
        elif v.startswith("[") and v.endswith("]"):
            cur[k] = [_parse_scalar(x) for x in v[1:-1].split(",") if x.strip()]
            key = None
        else:
            cur[k] = _parse_scalar(v)
            key = None
    return docs


def columns_from_docs(docs):
    """Documents -> name -> numpy array, as `Stream.from_loader`
    (psdfio.py:140-216) sets them: id, mass, time, position, velocity, and
    the acceleration, softening and potential where every document has
    them; a document without a type is a body."""
    for d in docs:
        t = d.get("type", "body")
        if t not in KINDS:
            raise ValueError("unknown particle type %r" % (t,))
        for k in ("id", "m", "t", "r", "v"):
            if k not in d:
                raise ValueError("particle document without %r" % k)
    cols = {"id": np.array([int(d["id"]) for d in docs], dtype=np.int64)}
    for key, name in SCALARS.items():
        if key == "id":
            continue
        if docs and all(key in d for d in docs):
            cols[name] = np.array([float(d[key]) for d in docs])
    for key, names in VECTORS.items():
        if docs and all(key in d for d in docs):
            vals = np.array([[float(x) for x in d[key]] for d in docs]).reshape(len(docs), 3)
            for j, nm in enumerate(names):
                cols[nm] = vals[:, j].copy()
    if not docs:
        for nm in ("mass", "time") + VECTORS["r"] + VECTORS["v"]:
            cols[nm] = np.zeros(0)
    return cols
