"""Reader of the reference's scene description files (.dl) into scenes.Scene.

The reference reads them with SceneReader (src/reader/SceneReader.cpp,
src/reader/DescriptionLanguage.cpp) into its scene graph and converts the
graph into an rt::Scene in MainWindow::convertScene (src/MainWindow.cpp:363-492).
This reader covers what the reference's scene files use:

- ``let NAME = value`` bindings, ``//`` comments;
- values: numbers, strings, vectors ``(a b c)``, dicts ``{key: value ...}``,
  lists ``[v v ...]``, member access ``Views.Up``, calls ``Get("name")``,
  ``From_sRGB(r g b)`` (0..255 sRGB to linear), ``*(a b)`` (product);
- ``Surface {name file}`` (a .be file relative to the .dl file),
  ``Material {name diffuse specular metalness roughness}``, ``Texture`` (ignored:
  environment textures are not part of the ray-patch path), ``Scene {...}``;
- scene objects with ``transform {position rotation scale}``, ``surface {model
  material}``, ``light {type color angle range}`` and child ``objects``.

The vector, quaternion and transform types come from the reference's
un-vendored Ds library, so their conventions are assumptions stated here:
rotations are Euler angles in degrees applied as R = Ry * Rx * Rz (about z,
then x, then y); a local transform is T * R * S and a child's world transform
is its parent's times its own; a light sits at its object's world position and
shines along the object's -z axis; the camera's vertical field of view is 60
degrees.  Light falloff is quadratic (the only one convertScene supports).
"""
from __future__ import annotations

import math
import os
import re

import numpy as np

from . import scenes as S

_TOKEN = re.compile(r"""
    (?P<ws>\s+|//[^\n]*) |
    (?P<num>[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?) |
    (?P<str>"[^"]*") |
    (?P<id>[A-Za-z_][A-Za-z_0-9]*) |
    (?P<op>[{}\[\]():.*=,])
""", re.VERBOSE)


def _tokens(text):
    pos = 0
    out = []
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise ValueError(f".dl: unexpected character {text[pos]!r} at offset {pos}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        v = m.group(kind)
        if kind == "num":
            out.append(("num", float(v) if any(c in v for c in ".eE") else int(v)))
        elif kind == "str":
            out.append(("str", v[1:-1]))
        else:
            out.append((kind, v))
    out.append(("eof", None))
    return out


class _Parser:
    def __init__(self, text, funcs, env):
        self.t = _tokens(text)
        self.i = 0
        self.funcs = funcs
        self.env = env

    def peek(self, k=0):
        return self.t[self.i + k]

    def take(self, kind=None, value=None):
        tok = self.t[self.i]
        if (kind and tok[0] != kind) or (value is not None and tok[1] != value):
            raise ValueError(f".dl: expected {value or kind}, found {tok[1]!r}")
        self.i += 1
        return tok

    def statements(self):
        while self.peek()[0] != "eof":
            tok = self.peek()
            if tok == ("id", "let"):
                self.take()
                name = self.take("id")[1]
                self.take("op", "=")
                self.env[name] = self.value()
            else:
                self.value()  # a top-level call such as Surface { ... }

    def value(self):
        kind, v = self.peek()
        if kind == "num":
            self.take()
            return v
        if kind == "str":
            self.take()
            return v
        if kind == "op" and v == "(":
            return self.vector()
        if kind == "op" and v == "{":
            return self.dict()
        if kind == "op" and v == "[":
            return self.list()
        if kind == "op" and v == "*":
            self.take()
            args = self.vector(raw=True)
            out = args[0]
            for a in args[1:]:
                out = np.asarray(out, np.float64) * np.asarray(a, np.float64)
            return out
        if kind == "id":
            self.take()
            if self.peek() == ("op", "("):
                args = self.vector(raw=True)
                return self.call(v, args)
            if self.peek() == ("op", "{"):
                return self.call(v, [self.dict()])
            out = self.env.get(v)
            if out is None:
                raise ValueError(f".dl: unknown name {v}")
            while self.peek() == ("op", "."):
                self.take()
                out = out[self.take("id")[1]]
            return out
        raise ValueError(f".dl: unexpected token {v!r}")

    def vector(self, raw=False):
        self.take("op", "(")
        items = []
        while self.peek() != ("op", ")"):
            items.append(self.value())
            if self.peek() == ("op", ","):
                self.take()
        self.take("op", ")")
        if raw:
            return items
        return np.asarray(items, np.float64) if items and all(np.isscalar(x) for x in items) else items

    def dict(self):
        self.take("op", "{")
        out = {}
        while self.peek() != ("op", "}"):
            key = self.take()[1]
            self.take("op", ":")
            out[key] = self.value()
            if self.peek() == ("op", ","):
                self.take()
        self.take("op", "}")
        return out

    def list(self):
        self.take("op", "[")
        out = []
        while self.peek() != ("op", "]"):
            out.append(self.value())
            if self.peek() == ("op", ","):
                self.take()
        self.take("op", "]")
        return out

    def call(self, name, args):
        fn = self.funcs.get(name)
        if fn is None:
            raise ValueError(f".dl: unknown function {name}")
        return fn(args)


def _srgb_to_linear(c):
    c = np.asarray(c, np.float64) / 255.0
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


def euler_matrix(deg):
    """R = Ry * Rx * Rz of Euler angles in degrees (the stated convention)."""
    x, y, z = (math.radians(float(a)) for a in deg)
    cx, sx, cy, sy, cz, sz = math.cos(x), math.sin(x), math.cos(y), math.sin(y), math.cos(z), math.sin(z)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return ry @ rx @ rz


def _quat_of(R):
    """Unit quaternion (x, y, z, w) of a rotation matrix."""
    t = R[0, 0] + R[1, 1] + R[2, 2]
    if t > 0:
        s = math.sqrt(t + 1.0) * 2
        w, x, y, z = 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        w, x, y, z = (R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s
    elif R[1, 1] > R[2, 2]:
        s = math.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        w, x, y, z = (R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s
    else:
        s = math.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        w, x, y, z = (R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s
    return tuple(float(np.float32(v)) for v in (x, y, z, w))


def _local(tr):
    M = np.eye(4)
    if not tr:
        return M
    S_ = np.diag(list(np.asarray(tr.get("scale", (1, 1, 1)), np.float64)) + [1.0])
    R = np.eye(4)
    R[:3, :3] = euler_matrix(tr.get("rotation", (0, 0, 0)))
    T = np.eye(4)
    T[:3, 3] = np.asarray(tr.get("position", (0, 0, 0)), np.float64)
    return T @ R @ S_


def load_dl(path: str, fovy_deg: float = 60.0):
    """Reads a .dl file.  Returns (scenes.Scene, scenes.Camera); surfaces are
    loaded from the .be files the file names, relative to it."""
    base = os.path.dirname(os.path.abspath(path))
    with open(path) as f:
        text = f.read()
    assets, materials = {}, {}
    surfaces, surface_index = [], {}
    state = {"scene": None}

    def surface(args):
        d = args[0]
        name = d.get("name", f"Surface_{len(assets)}")
        file = os.path.join(base, d["file"])
        assets[name] = ("surface", file)
        return assets[name]

    def material(args):
        d = args[0]
        name = d.get("name", f"Material_{len(materials)}")
        diff = tuple(float(v) for v in np.asarray(d.get("diffuse", (0.8, 0.8, 0.8)), np.float64))
        spec = tuple(float(v) for v in np.asarray(d.get("specular", (0.04, 0.04, 0.04)), np.float64))
        m = S.Material(tuple(float(np.float32(v)) for v in diff), tuple(float(np.float32(v)) for v in spec),
                       float(np.float32(d.get("metalness", 0.0))), float(np.float32(d.get("roughness", 0.5))))
        materials[name] = m
        assets[name] = ("material", m)
        return assets[name]

    def get(args):
        name = args[0]
        if name not in assets:
            raise ValueError(f".dl: unknown asset {name}")
        return assets[name]

    def scene(args):
        state["scene"] = args[0]
        return args[0]

    funcs = {"Surface": surface, "Material": material, "Get": get, "Scene": scene,
             "From_sRGB": lambda a: _srgb_to_linear(a), "Texture": lambda a: ("texture", None),
             "Mesh": lambda a: ("mesh", None)}
    _Parser(text, funcs, {}).statements()
    sc = state["scene"]
    if sc is None:
        raise ValueError(".dl: no Scene")

    objects, lights = [], []

    def surface_id(file):
        if file not in surface_index:
            surface_index[file] = len(surfaces)
            surfaces.append(S.load_be(file))
        return surface_index[file]

    def visit(obj, parent):
        world = parent @ _local(obj.get("transform"))
        srf = obj.get("surface")
        if srf and isinstance(srf.get("model"), tuple) and srf["model"][0] == "surface":
            sid = surface_id(srf["model"][1])
            mat = srf.get("material")
            m = mat[1] if isinstance(mat, tuple) and mat[0] == "material" else S.Material()
            l2w = world.astype(np.float64)
            objects.append(S.Object(sid, l2w.T.reshape(16).astype(np.float32),
                                    np.linalg.inv(l2w).T.reshape(16).astype(np.float32), m))
        li = obj.get("light")
        if li is not None:
            kind = li.get("type", "point")
            color = np.asarray(li.get("color", (1, 1, 1)), np.float64).reshape(-1)[:3]
            pos = world[:3, 3]
            dirn = -world[:3, 2]
            dirn = dirn / max(np.linalg.norm(dirn), 1e-30)
            angle = {"point": 3.1415, "directional": 0.0}.get(kind)
            if angle is None:
                angle = math.radians(float(li.get("angle", 45.0)))
            lights.append(S.Light(tuple(float(np.float32(c)) for c in color), 1.0,
                                  tuple(float(np.float32(c)) for c in pos), float(li.get("range", 0.0)),
                                  tuple(float(np.float32(c)) for c in dirn), angle))
        for child in obj.get("objects", []) or []:
            visit(child, world)

    for o in sc.get("objects", []) or []:
        visit(o, np.eye(4))
    env = sc.get("environment", {}) or {}
    bg = tuple(float(np.float32(v)) for v in np.asarray(env.get("background", (0.1, 0.1, 0.1)), np.float64))
    amb = tuple(float(np.float32(v)) for v in np.asarray(env.get("ambient", (0.1, 0.1, 0.1)), np.float64))
    view = sc.get("view", {}) or {}
    R = euler_matrix(view.get("rotation", (0, 0, 0)))
    cam = S.Camera(_quat_of(R), tuple(float(np.float32(v)) for v in np.asarray(view.get("position", (0, 0, 5)),
                                                                                np.float64)),
                   (1, 1, 1), float(np.float32(math.radians(fovy_deg))))
    scene_out = S.Scene(surfaces, objects, lights, bg, amb, name=os.path.basename(path))
    return scene_out, cam
