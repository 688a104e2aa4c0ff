"""Synthetic scenes of the trace-path workloads, written two ways.

Every scene is generated from a seeded NumPy PCG64 stream and can be emitted
as SDL (for the reference renderer, all numbers as round-trip literals) or as
a PovGpuSceneDesc (for libpovgpu and the oracle).  Both forms describe the
same parsed scene: the desc holds what the reference's parser leaves in
SceneData (camera vectors after Parse_Camera, plane Distance negated, finish
roughness inverted, mesh2 normals normalised), so the GPU path, the oracle
and the reference read identical values.

Workloads (names are descriptive, sizes are the defaults):
  spheres_plane   64 spheres + plane, 2 shadowing point lights, phong 0.5
                  (320x240, 1 spp, max_trace_level 1)
  mesh_spheres    1,051,392-triangle displaced sphere mesh2 + 1024 spheres +
                  plane, 1 light, reflection 0.3, max_trace_level 3
                  (1920x1080, 1 spp)
"""
import ctypes as C
import copy
import math

import numpy as np

from . import abi

EPSILON = 1.0e-10
M_PI_360 = 0.00872664625997164788


# ----------------------------------------------------------------- vectors --
def _sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def _scale(a, s):
    return (a[0] * s, a[1] * s, a[2] * s)


def _div(a, s):
    return (a[0] / s, a[1] / s, a[2] / s)


def _dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _cross(a, b):
    return ((a[1] * b[2]) - (a[2] * b[1]),
            (a[2] * b[0]) - (a[0] * b[2]),
            (a[0] * b[1]) - (a[1] * b[0]))


def _length(a):
    return math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])


def _normalized(a):
    l = _length(a)
    return _div(a, l) if l != 0 else a


def camera_vectors(location, look_at, angle, right_len, up_len=1.0, sky=(0.0, 1.0, 0.0)):
    """Camera vectors as Parse_Camera leaves them for
    ``camera { perspective location L look_at A angle a right x*r up y }``
    (source/parser/parser.cpp:1714-1790: angle first, then look_at)."""
    direction = (0.0, 0.0, 1.0)
    right = (right_len, 0.0, 0.0)
    up = (0.0, up_len, 0.0)
    # apply "angle"
    direction = _normalized(direction)
    right_length = _length(right)
    direction_length = right_length / math.tan(angle * M_PI_360) / 2.0
    direction = _scale(direction, direction_length)
    # apply "look_at"
    direction_length = _length(direction)
    up_length = _length(up)
    right_length = _length(right)
    handedness = _dot(_cross(up, direction), right)
    direction = _sub(look_at, location)
    direction = _normalized(direction)
    right = _cross(sky, direction)
    right = _normalized(right)
    up = _cross(direction, right)
    direction = _scale(direction, direction_length)
    right = _scale(right, right_length if handedness > 0.0 else -right_length)
    up = _scale(up, up_length)
    return direction, right, up


def _g(x):
    """Round-trip literal of a double."""
    return repr(float(x))


def _v(v):
    return "<%s,%s,%s>" % (_g(v[0]), _g(v[1]), _g(v[2]))


def _f32(x):
    """Round-trip literal of a float32 value (9 significant digits)."""
    return "%.9g" % float(x)


# -------------------------------------------------------------- transforms --
# TRANSFORM as the reference's parser builds it (source/core/math/matrix.cpp):
# row-vector convention (p' = p . M), `matrix` and `inverse` 4x4, composed
# by Compose_Transforms with the same multiplication order.
M_PI_180 = 0.01745329251994329576


def _identity():
    return [[1.0, 0.0, 0.0, 0.0], [0.0, 1.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0]]


def _mtimes_a(result, m2):
    """result = result x m2 (MTimesA, matrix.cpp:201)."""
    for i in range(4):
        t0, t1, t2, t3 = result[i]
        result[i] = [t0 * m2[0][j] + t1 * m2[1][j] + t2 * m2[2][j] + t3 * m2[3][j] for j in range(4)]


def _mtimes_b(m1, result):
    """result = m1 x result (MTimesB, matrix.cpp:242)."""
    for j in range(4):
        t0, t1, t2, t3 = result[0][j], result[1][j], result[2][j], result[3][j]
        for i in range(4):
            result[i][j] = m1[i][0] * t0 + m1[i][1] * t1 + m1[i][2] * t2 + m1[i][3] * t3


def _transpose(m):
    return [[m[j][i] for j in range(4)] for i in range(4)]


class Transform:
    def __init__(self):
        self.matrix = _identity()
        self.inverse = _identity()

    @staticmethod
    def rotation(v):
        """Compute_Rotation_Transform (matrix.cpp:685-737)."""
        t = Transform()
        rx, ry, rz = (float(v[0]) * M_PI_180, float(v[1]) * M_PI_180, float(v[2]) * M_PI_180)
        cx, sx, cy, sy, cz, sz = math.cos(rx), math.sin(rx), math.cos(ry), math.sin(ry), math.cos(rz), math.sin(rz)
        t.matrix[1][1] = cx
        t.matrix[2][2] = cx
        t.matrix[1][2] = sx
        t.matrix[2][1] = 0.0 - sx
        t.inverse = _transpose(t.matrix)
        m = _identity()
        m[0][0] = cy
        m[2][2] = cy
        m[0][2] = 0.0 - sy
        m[2][0] = sy
        _mtimes_a(t.matrix, m)
        _mtimes_b(_transpose(m), t.inverse)
        m = _identity()
        m[0][0] = cz
        m[1][1] = cz
        m[0][1] = sz
        m[1][0] = 0.0 - sz
        _mtimes_a(t.matrix, m)
        _mtimes_b(_transpose(m), t.inverse)
        return t

    @staticmethod
    def scaling(v):
        """Compute_Scaling_Transform (matrix.cpp:596-612)."""
        t = Transform()
        for k in range(3):
            t.matrix[k][k] = float(v[k])
            t.inverse[k][k] = 1.0 / float(v[k])
        return t

    @staticmethod
    def translation(v):
        """Compute_Translation_Transform (matrix.cpp:644-657)."""
        t = Transform()
        t.matrix[3][0], t.matrix[3][1], t.matrix[3][2] = float(v[0]), float(v[1]), float(v[2])
        t.inverse[3][0], t.inverse[3][1], t.inverse[3][2] = -float(v[0]), -float(v[1]), -float(v[2])
        return t

    def compose(self, add):
        """Compose_Transforms (matrix.cpp:788-793)."""
        _mtimes_a(self.matrix, add.matrix)
        _mtimes_b(add.inverse, self.inverse)
        return self

    def flat(self):
        return [x for row in self.matrix for x in row] + [x for row in self.inverse for x in row]


# ------------------------------------------------------------------ scenes --
class Pattern:
    """A pattern pigment: `kind` one of checker, gradient, bozo, spotted,
    granite, marble, wood, agate, onion, leopard; `colours` the colour map
    as [(value, rgb), ...] (checker: its two colours as [(0, rgb_a),
    (1, rgb_b)]); `transforms` the pigment's transformations in SDL order,
    each ("scale" | "rotate" | "translate", vector); `gradient` the gradient
    pattern's vector; `noise_generator` 1-3 or None for the scene's default
    (2, range corrected); `turbulence` the classic turbulence vector (None:
    no turbulence; agate always has one) with `octaves`, `omega`, `lambda_`;
    `wave` one of ramp, sine, triangle, scallop, cubic, poly (None: the
    pattern's default) with `frequency`, `phase`, `exponent`; `agate_turb`."""
    KINDS = {"checker": abi.POV_PATTERN_CHECKER, "gradient": abi.POV_PATTERN_GRADIENT,
             "bozo": abi.POV_PATTERN_BOZO, "spotted": abi.POV_PATTERN_BOZO, "granite": abi.POV_PATTERN_GRANITE,
             "marble": abi.POV_PATTERN_MARBLE, "wood": abi.POV_PATTERN_WOOD, "agate": abi.POV_PATTERN_AGATE,
             "onion": abi.POV_PATTERN_ONION, "leopard": abi.POV_PATTERN_LEOPARD,
             # normal-only patterns
             "bumps": abi.POV_PATTERN_BUMPS, "dents": abi.POV_PATTERN_DENTS,
             "wrinkles": abi.POV_PATTERN_WRINKLES,
             # pigment or normal
             "ripples": abi.POV_PATTERN_RIPPLES, "waves": abi.POV_PATTERN_WAVES,
             "radial": abi.POV_PATTERN_RADIAL, "planar": abi.POV_PATTERN_PLANAR,
             "spherical": abi.POV_PATTERN_SPHERICAL, "cylindrical": abi.POV_PATTERN_CYLINDRICAL,
             "boxed": abi.POV_PATTERN_BOXED,
             # discrete, with a colour list of 4, 6 and 6 entries at 0..n-1
             "square": abi.POV_PATTERN_SQUARE, "triangular": abi.POV_PATTERN_TRIANGULAR,
             "cubic": abi.POV_PATTERN_CUBIC, "hexagon": abi.POV_PATTERN_HEXAGON,
             # brick (discrete: mortar, brick), spiral1 / spiral2 (`arms`), cells
             "brick": abi.POV_PATTERN_BRICK, "spiral1": abi.POV_PATTERN_SPIRAL1,
             "spiral2": abi.POV_PATTERN_SPIRAL2, "cells": abi.POV_PATTERN_CELLS,
             # crackle (form, metric, offset, solid), quilted (control0/1; pigment only)
             "crackle": abi.POV_PATTERN_CRACKLE, "quilted": abi.POV_PATTERN_QUILTED}
    DISCRETE = ("checker", "square", "triangular", "cubic", "hexagon", "brick")

    def __init__(self, kind, colours, transforms=(), gradient=(1.0, 0.0, 0.0), noise_generator=None,
                 turbulence=None, octaves=6, omega=0.5, lambda_=2.0, wave=None, frequency=1.0, phase=0.0,
                 exponent=1.0, agate_turb=1.0, brick_size=(8.0, 3.0, 4.5), mortar=0.5, arms=3,
                 form=None, metric=None, offset=None, solid=False, control0=None, control1=None):
        assert kind in self.KINDS
        self.form = None if form is None else tuple(float(x) for x in form)
        self.metric = None if metric is None else float(metric)
        self.offset = None if offset is None else float(offset)
        self.solid = bool(solid)
        self.control0 = None if control0 is None else float(control0)
        self.control1 = None if control1 is None else float(control1)
        self.brick_size = tuple(float(x) for x in brick_size)
        self.mortar = float(mortar)
        self.arms = int(arms)
        self.kind = kind
        # entries (value, rgb) or (value, rgb, filter, transmit)
        self.colours = [(float(e[0]), tuple(float(c) for c in e[1])) for e in colours]
        self.ft = [(float(e[2]), float(e[3])) if len(e) > 2 else (0.0, 0.0) for e in colours]
        self.transforms = [(op, tuple(float(x) for x in vec)) for op, vec in transforms]
        self.gradient = tuple(float(x) for x in gradient)
        self.noise_generator = noise_generator
        self.turbulence = None if turbulence is None else tuple(float(x) for x in turbulence)
        self.octaves, self.omega, self.lambda_ = int(octaves), float(omega), float(lambda_)
        self.wave = wave
        self.frequency, self.phase, self.exponent = float(frequency), float(phase), float(exponent)
        self.frequency_default = frequency == 1.0   # no frequency in the SDL: the pattern's default
        self.agate_turb = float(agate_turb)

    def sdl(self, amount=None):
        """The pigment body; with `amount`, the body of a normal of that
        amount (no colour map, the amount right after the pattern)."""
        if self.kind in self.DISCRETE:
            body = self.kind + "".join(" color %s" % self._colour(k) for k in range(len(self.colours)))
            if self.kind == "brick":
                body += " brick_size %s mortar %s" % (_v(self.brick_size), _g(self.mortar))
        else:
            head = "gradient %s" % _v(self.gradient) if self.kind == "gradient" else self.kind
            if self.kind in ("spiral1", "spiral2"):
                head += " %d" % self.arms
            if amount is not None:
                body = "%s, %s" % (head, _g(amount))
            else:
                cmap = " ".join("[%s color %s]" % (_f32(v), self._colour(k)) for k, (v, _c) in enumerate(self.colours))
                body = "%s color_map { %s }" % (head, cmap)
            if self.kind == "agate" and self.agate_turb != 1.0:
                body += " agate_turb %s" % _g(self.agate_turb)
            if self.form is not None:
                body += " form %s" % _v(self.form)
            if self.metric is not None:
                body += " metric %s" % _g(self.metric)
            if self.offset is not None:
                body += " offset %s" % _g(self.offset)
            if self.solid:
                body += " solid"
            if self.control0 is not None:
                body += " control0 %s" % _g(self.control0)
            if self.control1 is not None:
                body += " control1 %s" % _g(self.control1)
            if self.wave is not None:
                body += " %s_wave" % self.wave if self.wave != "poly" else " poly_wave %s" % _g(self.exponent)
            if self.frequency != 1.0:
                body += " frequency %s" % _g(self.frequency)
            if self.phase != 0.0:
                body += " phase %s" % _g(self.phase)
        if self.noise_generator is not None:
            body += " noise_generator %d" % self.noise_generator
        if self.turbulence is not None:
            body += " turbulence %s octaves %d omega %s lambda %s" % (_v(self.turbulence), self.octaves,
                                                                      _g(self.omega), _g(self.lambda_))
        for op, vec in self.transforms:
            body += " %s %s" % (op, _v(vec))
        return body

    def _colour(self, k):
        c = self.colours[k][1]
        f, t = self.ft[k]
        if f or t:
            return "rgbft <%s,%s,%s,%s,%s>" % (_g(c[0]), _g(c[1]), _g(c[2]), _g(f), _g(t))
        return "rgb %s" % _v(c)

    def transparent(self):
        return any(f or t for f, t in self.ft)

    def transform(self):
        t = Transform()
        for op, vec in self.transforms:
            t.compose({"scale": Transform.scaling, "rotate": Transform.rotation,
                       "translate": Transform.translation}[op](vec))
        return t

    def desc(self):
        d = abi.PovGpuPattern()
        d.type = self.KINDS[self.kind]
        d.noise_generator = 2 if self.noise_generator is None else int(self.noise_generator)
        d.num_entries = len(self.colours)
        default_wave = "triangle" if self.kind in ("marble", "wood", "spiral1", "spiral2") else "ramp"
        d.wave_type = abi.POV_WAVES[self.wave or default_wave]
        inv = self.transform().inverse
        for i in range(4):
            for j in range(4):
                d.inverse[4 * i + j] = inv[i][j]
        # the parser normalises the gradient vector (parser_materials.cpp:1443)
        gl = math.sqrt(sum(x * x for x in self.gradient))
        d.gradient[:] = tuple(x / gl for x in self.gradient) if gl > 0.0 else self.gradient
        d.frequency, d.phase, d.exponent = self.frequency, self.phase, self.exponent
        turb = self.turbulence
        # agate always carries a classic turbulence warp (Check_Turb in the parser)
        d.has_turbulence = 1 if (turb is not None or self.kind == "agate") else 0
        d.turbulence[:] = turb if turb is not None else (0.0, 0.0, 0.0)
        d.omega = self.omega
        setattr(d, "lambda", self.lambda_)
        d.octaves = self.octaves
        d.agate_turb = self.agate_turb
        d.brick_size[:] = self.brick_size
        d.mortar = float(np.float32(self.mortar - 2.0e-10))   # SNGL, less EPSILON * 2 (parser_materials.cpp:2062)
        d.arms = self.arms
        d.crackle_form[:] = self.form if self.form is not None else (-1.0, 1.0, 0.0)
        d.crackle_metric = 2.0 if self.metric is None else self.metric
        d.crackle_offset = 0.0 if self.offset is None else self.offset
        d.crackle_solid = int(self.solid)
        d.control0 = float(np.float32(1.0 if self.control0 is None else self.control0))   # SNGL
        d.control1 = float(np.float32(1.0 if self.control1 is None else self.control1))
        if self.kind == "quilted" and self.frequency_default:
            d.frequency = 0.0   # QuiltedPattern's default (pattern.cpp:667)
        for k, (v, c) in enumerate(self.colours):
            d.values[k] = v
            d.colours[k][:] = c
            d.filters[k], d.transmits[k] = self.ft[k]
        return d


class Normal:
    """A normal perturbation: `pattern` a Pattern whose kind is bumps, dents,
    wrinkles or a continuous pattern (gradient, bozo, spotted, granite,
    marble, wood, agate, onion, leopard; no colour map needed), `amount`
    (0.5 by default), `accuracy` (the slope's delta, 0.02 by default) and
    `no_bump_scale`."""

    def __init__(self, pattern, amount=0.5, accuracy=0.02, no_bump_scale=False):
        assert pattern.kind not in Pattern.DISCRETE
        self.pattern = pattern
        self.amount = float(amount)
        self.accuracy = float(accuracy)
        self.no_bump_scale = bool(no_bump_scale)

    def sdl(self):
        body = self.pattern.sdl(amount=self.amount)
        if self.accuracy != 0.02:
            body += " accuracy %s" % _g(self.accuracy)
        if self.no_bump_scale:
            body += " no_bump_scale"
        return body

    def desc(self, pattern_index):
        d = abi.PovGpuNormal()
        d.pattern = pattern_index
        d.dont_scale_bumps = 1 if self.no_bump_scale else 0
        d.amount = self.amount
        d.delta = self.accuracy
        fwd = self.pattern.transform().matrix
        for i in range(4):
            for j in range(4):
                d.matrix[4 * i + j] = fwd[i][j]
        return d


class Material:
    def __init__(self, rgb, ambient=0.1, diffuse=0.6, phong=0.0, phong_size=40.0,
                 specular=0.0, roughness=0.05, reflection=0.0, brilliance=1.0,
                 emission=0.0, transmit=0.0, pattern=None, normal=None, filter=0.0,
                 reflection_min=None, fresnel=False, conserve_energy=False, diffuse_back=0.0, metallic=0.0,
                 reflect_metallic=0.0):
        """`reflection` alone is the old syntax (min = max); with
        `reflection_min` or `fresnel` the finish takes the block form
        reflection { min, max fresnel } (Parse_Finish,
        source/parser/parser_materials.cpp:2288-2348).  conserve_energy:
        the transmitted light loses what the surface reflects."""
        self.diffuse_back = float(diffuse_back)   # `diffuse A, B`: B lights the back side
        self.metallic = float(metallic)           # finish { metallic m }: tinted highlights
        self.reflect_metallic = float(reflect_metallic)   # reflection { ... metallic m }
        self.reflection_min = None if reflection_min is None else float(reflection_min)
        self.fresnel = bool(fresnel)
        self.conserve_energy = bool(conserve_energy)
        self.pattern = pattern
        self.normal = normal
        self.rgb = tuple(float(c) for c in rgb)
        self.transmit = float(transmit)
        self.filter = float(filter)
        self.ambient = float(ambient)
        self.diffuse = float(diffuse)
        self.phong = float(phong)
        self.phong_size = float(phong_size)
        self.specular = float(specular)
        self.roughness = float(roughness)
        self.reflection = float(reflection)
        self.brilliance = float(brilliance)
        self.emission = float(emission)

    def sdl(self):
        fin = "ambient %s diffuse %s" % (_g(self.ambient), _g(self.diffuse))
        if self.diffuse_back:
            fin += ", %s" % _g(self.diffuse_back)
        if self.brilliance != 1.0:
            fin += " brilliance %s" % _g(self.brilliance)
        if self.phong:
            fin += " phong %s phong_size %s" % (_g(self.phong), _g(self.phong_size))
        if self.specular:
            fin += " specular %s roughness %s" % (_g(self.specular), _g(self.roughness))
        if self.metallic:
            fin += " metallic %s" % _g(self.metallic)
        if self.reflection_min is not None or self.fresnel or self.reflect_metallic:
            rmin = self.reflection if self.reflection_min is None else self.reflection_min
            fin += " reflection { %s, %s%s%s }" % (_g(rmin), _g(self.reflection), " fresnel on" if self.fresnel else "",
                                                  " metallic %s" % _g(self.reflect_metallic)
                                                  if self.reflect_metallic else "")
        elif self.reflection:
            fin += " reflection %s" % _g(self.reflection)
        if self.conserve_energy:
            fin += " conserve_energy"
        if self.emission:
            fin += " emission %s" % _g(self.emission)
        if self.pattern is not None:
            pig = self.pattern.sdl()
        elif self.filter:
            pig = "color rgbft <%s,%s,%s,%s,%s>" % (_g(self.rgb[0]), _g(self.rgb[1]), _g(self.rgb[2]),
                                                   _g(self.filter), _g(self.transmit))
        elif self.transmit:
            pig = "color rgbt <%s,%s,%s,%s>" % (_g(self.rgb[0]), _g(self.rgb[1]), _g(self.rgb[2]), _g(self.transmit))
        else:
            pig = "color rgb %s" % _v(self.rgb)
        nrm = "" if self.normal is None else " normal { %s }" % self.normal.sdl()
        return "texture { pigment { %s }%s finish { %s } }" % (pig, nrm, fin)

    def desc(self):
        m = abi.PovGpuMaterial()
        m.pigment[:] = [self.rgb[0], self.rgb[1], self.rgb[2], self.filter, self.transmit]
        m.ambient[:] = [self.ambient] * 3
        m.emission[:] = [self.emission] * 3
        m.diffuse = self.diffuse
        m.diffuse_back = self.diffuse_back
        m.brilliance = self.brilliance
        m.brilliance_adjust = 1.0
        m.brilliance_adjust_rad = 2.0 / (self.brilliance + 1.0)
        m.phong = self.phong
        m.phong_size = self.phong_size
        m.specular = self.specular
        m.roughness = 1.0 / self.roughness
        m.metallic = self.metallic
        m.reflection_max[:] = [self.reflection] * 3
        m.reflection_min[:] = [self.reflection if self.reflection_min is None else self.reflection_min] * 3
        m.reflection_falloff = 1.0
        m.reflect_exp = 1.0
        m.reflect_metallic = self.reflect_metallic
        m.reflection_fresnel = int(self.fresnel)
        m.conserve_energy = int(self.conserve_energy)
        m.fresnel = 0.0
        m.crand = 0.0
        m.irid = 0.0
        return m


class Interior:
    """interior { ior fade_distance fade_power fade_color } of an object
    (Parse_Interior, source/parser/parser_materials.cpp); the defaults are
    the parser's (Interior::Interior, source/core/material/interior.cpp:
    58-73, with IOR 0 replaced by the atmosphere's 1.0 in Post_Process)."""

    def __init__(self, ior=1.0, fade_distance=0.0, fade_power=0.0, fade_colour=(0.0, 0.0, 0.0)):
        self.ior = float(ior)
        self.fade_distance = float(fade_distance)
        self.fade_power = float(fade_power)
        self.fade_colour = tuple(float(c) for c in fade_colour)

    def sdl(self):
        out = "interior { ior %s" % _g(self.ior)
        if self.fade_distance or self.fade_power:
            out += " fade_distance %s fade_power %s fade_color rgb %s" % (
                _g(self.fade_distance), _g(self.fade_power), _v(self.fade_colour))
        return out + " }"

    def desc(self):
        d = abi.PovGpuInterior()
        d.ior = self.ior
        d.dispersion = 1.0
        d.caustics = 0.0
        d.fade_distance = self.fade_distance
        d.fade_power = self.fade_power
        d.fade_colour[:] = list(self.fade_colour)
        d.old_refract = 1.0
        return d


class Mesh:
    """mesh2 with per-vertex normals (normal_indices = face_indices)."""

    def __init__(self, vertices, normals, faces):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32)
        self.normals = None if normals is None else np.ascontiguousarray(normals, dtype=np.float32)
        self.faces = np.ascontiguousarray(faces, dtype=np.int32)

    @property
    def num_triangles(self):
        return int(self.faces.shape[0])

    def sdl(self, material):
        out = ["mesh2 {\n  vertex_vectors { %d,\n" % len(self.vertices)]
        out.append(",\n".join("<%s,%s,%s>" % (_f32(a), _f32(b), _f32(c)) for a, b, c in self.vertices))
        out.append("\n  }\n")
        if self.normals is not None:
            out.append("  normal_vectors { %d,\n" % len(self.normals))
            out.append(",\n".join("<%s,%s,%s>" % (_f32(a), _f32(b), _f32(c)) for a, b, c in self.normals))
            out.append("\n  }\n")
        out.append("  face_indices { %d,\n" % len(self.faces))
        out.append(",\n".join("<%d,%d,%d>" % (a, b, c) for a, b, c in self.faces))
        out.append("\n  }\n")
        out.append("  %s\n}\n" % material.sdl())
        return "".join(out)


class Scene:
    def __init__(self, name, width, height, location, look_at, angle,
                 max_trace_level=5, adc_bailout=1.0 / 255.0, background=(0.0, 0.0, 0.0)):
        self.name = name
        self.width = int(width)
        self.height = int(height)
        self.location = tuple(float(x) for x in location)
        self.look_at = tuple(float(x) for x in look_at)
        self.angle = float(angle)
        self.right_len = float(width) / float(height)
        self.max_trace_level = int(max_trace_level)
        self.adc_bailout = float(adc_bailout)
        self.background = tuple(float(x) for x in background)
        self.materials = []
        self.objects = []     # list of dicts, depth-first order
        self.lights = []
        self.meshes = []
        self.antialias = None  # (threshold, depth) for sampling method 2
        self.radiosity = None  # dict of radiosity{} settings, None = off
        self.medias = []       # interior media of container objects

    # -- building ----------------------------------------------------------
    def material(self, m):
        self.materials.append(m)
        return len(self.materials) - 1

    def sphere(self, centre, radius, mat, interior=None):
        self.objects.append(dict(type=abi.POV_OBJ_SPHERE, centre=tuple(map(float, centre)),
                                 radius=float(radius), material=mat, interior=interior))

    def plane(self, normal, offset, mat):
        self.objects.append(dict(type=abi.POV_OBJ_PLANE, normal=tuple(map(float, normal)),
                                 offset=float(offset), material=mat))

    def mesh(self, mesh, mat):
        self.meshes.append(mesh)
        self.objects.append(dict(type=abi.POV_OBJ_MESH, mesh=len(self.meshes) - 1, material=mat))

    def add(self, node):
        """Adds an object tree built with the node helpers below."""
        self.objects.append(node)

    # node helpers (material -1 = inherited from the enclosing CSG)
    @staticmethod
    def n_sphere(centre, radius, mat=-1, interior=None):
        return dict(type=abi.POV_OBJ_SPHERE, centre=tuple(map(float, centre)), radius=float(radius), material=mat,
                    interior=interior)

    @staticmethod
    def n_box(c1, c2, mat=-1, interior=None):
        lo = tuple(min(float(a), float(b)) for a, b in zip(c1, c2))
        hi = tuple(max(float(a), float(b)) for a, b in zip(c1, c2))
        return dict(type=abi.POV_OBJ_BOX, c1=lo, c2=hi, material=mat, interior=interior)

    @staticmethod
    def n_torus(major, minor, rotate=(0.0, 0.0, 0.0), translate=(0.0, 0.0, 0.0), mat=-1):
        t = Transform().compose(Transform.rotation(rotate)).compose(Transform.translation(translate))
        return dict(type=abi.POV_OBJ_TORUS, R=float(major), r=float(minor), trans=t,
                    mods="rotate %s translate %s" % (_v(rotate), _v(translate)), material=mat)

    @staticmethod
    def n_csg(kind, children, translate=(0.0, 0.0, 0.0), mat=-1, interior=None):
        """kind: 'union', 'intersection', 'difference' or 'merge'.  The
        translation is applied to the children as the parser does
        (Sphere/Box::Translate move the geometry; CSG::Translate recurses)."""
        tv = tuple(map(float, translate))
        moved = []
        for c in children:
            c = dict(c)
            if c["type"] == abi.POV_OBJ_SPHERE:
                c["sdl_centre"] = c["centre"]
                c["centre"] = tuple(a + b for a, b in zip(c["centre"], tv))
            elif c["type"] == abi.POV_OBJ_BOX:
                c["sdl_c1"], c["sdl_c2"] = c["c1"], c["c2"]
                c["c1"] = tuple(a + b for a, b in zip(c["c1"], tv))
                c["c2"] = tuple(a + b for a, b in zip(c["c2"], tv))
            elif not (c["type"] == abi.POV_OBJ_TORUS and tv == (0.0, 0.0, 0.0)):
                raise ValueError("CSG children: spheres and boxes (tori in an untranslated CSG)")
            moved.append(c)
        if kind == "difference":
            for c in moved[1:]:
                c["inverted"] = True
        t = {"union": abi.POV_OBJ_UNION, "intersection": abi.POV_OBJ_INTERSECTION,
             "difference": abi.POV_OBJ_INTERSECTION, "merge": abi.POV_OBJ_MERGE}[kind]
        return dict(type=t, kind=kind, children=moved, translate=tv, material=mat, interior=interior)

    def media_box(self, c1, c2, scattering=(0.05, 0.05, 0.05), absorption=(0.0, 0.0, 0.0),
                  emission=(0.0, 0.0, 0.0), intervals=10, samples=10, aa_level=3, aa_threshold=0.1,
                  scattering_type=1, eccentricity=0.0, sphere=None):
        """A hollow, fully transmitting box holding one uniform media
        (Parse_Media defaults, source/parser/parser_materials.cpp:3500-3630:
        method 3, jitter 0; Media::PostProcess sets extinction = absorption +
        scattering).  scattering_type: 1 isotropic, 2 Mie hazy, 3 Mie murky,
        4 Rayleigh, 5 Henyey-Greenstein with `eccentricity`.  `sphere`
        (centre, radius): a hollow sphere holds the media instead of the box
        c1, c2."""
        mat = self.material(Material((1.0, 1.0, 1.0), ambient=0.0, diffuse=0.0, transmit=1.0))
        self.medias.append(dict(scattering=tuple(map(float, scattering)), absorption=tuple(map(float, absorption)),
                                emission=tuple(map(float, emission)), intervals=int(intervals),
                                samples=int(samples), aa_level=int(aa_level), aa_threshold=float(aa_threshold),
                                scattering_type=int(scattering_type), eccentricity=float(eccentricity)))
        if sphere is not None:   # a sphere container: centre, radius
            node = dict(type=abi.POV_OBJ_SPHERE, centre=tuple(map(float, sphere[0])), radius=float(sphere[1]),
                        material=mat, interior=None)
        else:
            node = self.n_box(c1, c2, mat)
        node["hollow"] = True
        node["media"] = len(self.medias)
        self.objects.append(node)

    def point_light(self, pos, rgb=(1.0, 1.0, 1.0)):
        self.lights.append(dict(kind=abi.POV_LIGHT_POINT, pos=tuple(map(float, pos)),
                                rgb=tuple(map(float, rgb))))

    def light(self, pos, rgb=(1.0, 1.0, 1.0), beam=None, point_at=None, radius=None, falloff=None,
              tightness=None, parallel=False, shadowless=False, fade_distance=None, fade_power=None):
        """light_source with the modifiers of Parse_Light_Source
        (source/parser/parser.cpp:3345-3406), written in this order: `beam`
        "spotlight" or "cylinder" (their defaults: radius 30 / falloff 45
        degrees, tightness 0; radius 0.75, falloff 1, tightness 0 and
        parallel), radius, falloff, tightness, parallel, point_at,
        shadowless (which makes the light a fill light whatever came
        before), fade_distance, fade_power.  A spotlight's radius and
        falloff are angles in degrees, a cylinder's lengths."""
        l = dict(kind=abi.POV_LIGHT_POINT, pos=tuple(map(float, pos)), rgb=tuple(map(float, rgb)),
                 beam=beam, point_at=None if point_at is None else tuple(map(float, point_at)),
                 radius=radius, falloff=falloff, tightness=tightness, parallel=bool(parallel),
                 shadowless=bool(shadowless), fade_distance=fade_distance, fade_power=fade_power)
        if beam not in (None, "spotlight", "cylinder"):
            raise ValueError("beam: None, 'spotlight' or 'cylinder'")
        self.lights.append(l)
        return l

    @staticmethod
    def _light_fields(l):
        """The LightSource fields the parser leaves for light dict `l`
        (Parse_Light_Source, LightSource::LightSource defaults,
        lightsource.cpp:355-400): light_type, parallel, points_at, radius,
        falloff, tightness, fade_distance, fade_power."""
        f = dict(light_type=1, parallel=False, points_at=(0.0, 0.0, 1.0), radius=0.0, falloff=0.0,
                 tightness=0.0, fade_distance=0.0, fade_power=0.0)
        deg = 0.01745329251994329576   # M_PI_180
        if l.get("beam") == "spotlight":
            f.update(light_type=2, radius=math.cos(30 * deg), falloff=math.cos(45 * deg))
        elif l.get("beam") == "cylinder":
            f.update(light_type=4, radius=0.75, falloff=1.0, parallel=True)
        spot = f["light_type"] == 2
        if l.get("radius") is not None:
            f["radius"] = math.cos(float(l["radius"]) * deg) if spot else float(l["radius"])
        if l.get("falloff") is not None:
            f["falloff"] = math.cos(float(l["falloff"]) * deg) if spot else float(l["falloff"])
        if l.get("tightness") is not None:
            f["tightness"] = float(l["tightness"])
        if l.get("point_at") is not None:
            f["points_at"] = l["point_at"]
        if l.get("parallel"):
            f["parallel"] = True
        if l.get("shadowless"):
            f["light_type"] = 3
        if l.get("fade_distance") is not None:
            f["fade_distance"] = float(l["fade_distance"])
        if l.get("fade_power") is not None:
            f["fade_power"] = float(l["fade_power"])
        # legacy (pre-3.8) scenes ignore fade_power without fade_distance
        # (parser.cpp:3508-3513); the SDL here is #version 3.7
        if f["fade_power"] != 0 and abs(f["fade_distance"]) < 1e-10:
            f["fade_power"] = f["fade_distance"] = 0.0
        return f

    @staticmethod
    def _light_sdl(l):
        out = ""
        if l.get("beam") is not None:
            out += " " + l["beam"]
        for key in ("radius", "falloff", "tightness"):
            if l.get(key) is not None:
                out += " %s %s" % (key, _g(l[key]))
        if l.get("parallel"):
            out += " parallel"
        if l.get("point_at") is not None:   # after spotlight, cylinder or parallel (parser.cpp:3368-3377)
            out += " point_at %s" % _v(l["point_at"])
        if l.get("shadowless"):
            out += " shadowless"
        for key in ("fade_distance", "fade_power"):
            if l.get(key) is not None:
                out += " %s %s" % (key, _g(l[key]))
        return out

    def area_light(self, pos, axis1, axis2, size1, size2, rgb=(1.0, 1.0, 1.0), adaptive=None,
                   circular=False, orient=False):
        """light_source with area_light (Parse_Light_Source,
        source/parser/parser.cpp:3421-3467); `adaptive` None keeps the
        parser's default Adaptive_Level 100 (lightsource.cpp:392).  The
        post-parse rules apply: orient implies circular, and circular needs
        more than one sample per axis (parser.cpp:9156-9192)."""
        size1, size2 = int(size1), int(size2)
        if size1 < 1 or size2 < 1:
            raise ValueError("Area size must be greater than zero.")
        circular = bool(circular) or bool(orient)
        if circular and (size1 <= 1 or size2 <= 1):
            circular = False
        self.lights.append(dict(kind=abi.POV_LIGHT_AREA, pos=tuple(map(float, pos)),
                                rgb=tuple(map(float, rgb)), axis1=tuple(map(float, axis1)),
                                axis2=tuple(map(float, axis2)), size=(size1, size2),
                                adaptive=adaptive, circular=circular, orient=bool(orient)))

    # -- SDL -----------------------------------------------------------------
    def sdl(self):
        rad = ""
        if self.radiosity is not None:
            r = self.radiosity_settings()
            rad = (" radiosity { count %d recursion_limit %d error_bound %s nearest_count %d"
                   " pretrace_start %s pretrace_end %s minimum_reuse %s maximum_reuse %s"
                   " low_error_factor %s gray_threshold %s brightness %s adc_bailout %s }"
                   % (r["count"], r["recursion_limit"], _g(r["error_bound"]), r["nearest_count"],
                      _g(r["pretrace_start"]), _g(r["pretrace_end"]), _g(r["minimum_reuse"]),
                      _g(r["maximum_reuse"]), _g(r["low_error_factor"]), _g(r["gray_threshold"]),
                      _g(r["brightness"]), _g(r["adc_bailout"])))
        out = ["#version 3.7;\n",
               "global_settings { assumed_gamma 1.0 max_trace_level %d adc_bailout %s%s }\n"
               % (self.max_trace_level, _g(self.adc_bailout), rad),
               "camera { perspective location %s right x*%s up y look_at %s angle %s }\n"
               % (_v(self.location), _g(self.right_len), _v(self.look_at), _g(self.angle)),
               "background { color rgb %s }\n" % _v(self.background)]
        for l in self.lights:
            extra = ""
            if l["kind"] == abi.POV_LIGHT_AREA:
                extra = " area_light %s, %s, %d, %d" % (_v(l["axis1"]), _v(l["axis2"]), l["size"][0], l["size"][1])
                if l["adaptive"] is not None:
                    extra += " adaptive %d" % l["adaptive"]
                if l["circular"]:
                    extra += " circular"
                if l["orient"]:
                    extra += " orient"
            extra += self._light_sdl(l)
            out.append("light_source { %s color rgb %s%s }\n" % (_v(l["pos"]), _v(l["rgb"]), extra))
        for o in self.objects:
            out.append(self._sdl_node(o) + "\n")
        return "".join(out)

    def radiosity_settings(self):
        """The radiosity{} block with the parser's defaults filled in
        (SceneRadiositySettings, source/core/lighting/radiosity.h:137-165)."""
        r = dict(count=35, recursion_limit=2, error_bound=1.8, nearest_count=5, pretrace_start=0.08,
                 pretrace_end=0.04, minimum_reuse=0.015, maximum_reuse=0.2, low_error_factor=0.5,
                 gray_threshold=0.0, brightness=1.0, adc_bailout=0.01, always_sample=False)
        r.update(self.radiosity or {})
        return r

    def _media_sdl(self, o):
        """`hollow` and the interior media of a container object."""
        extra = ""
        if o.get("hollow"):
            extra += " hollow"
        if o.get("media"):
            md = self.medias[o["media"] - 1]
            ecc = (" eccentricity %s" % _g(md["eccentricity"])) if md["scattering_type"] == 5 else ""
            extra += (" interior { media { scattering { %d, rgb %s%s } absorption rgb %s emission rgb %s"
                      " intervals %d samples %d aa_level %d aa_threshold %s } }"
                      % (md["scattering_type"], _v(md["scattering"]), ecc, _v(md["absorption"]),
                         _v(md["emission"]), md["intervals"], md["samples"], md["aa_level"], _g(md["aa_threshold"])))
        return extra

    def _sdl_node(self, o):
        tex = (" " + self.materials[o["material"]].sdl()) if o.get("material", -1) >= 0 else ""
        if o.get("interior") is not None:
            tex += " " + o["interior"].sdl()
        t = o["type"]
        if t == abi.POV_OBJ_SPHERE:
            return "sphere { %s, %s%s%s }" % (_v(o.get("sdl_centre", o["centre"])), _g(o["radius"]), tex,
                                              self._media_sdl(o))
        if t == abi.POV_OBJ_PLANE:
            return "plane { %s, %s%s }" % (_v(o["normal"]), _g(o["offset"]), tex)
        if t == abi.POV_OBJ_BOX:
            return "box { %s, %s%s%s }" % (_v(o.get("sdl_c1", o["c1"])), _v(o.get("sdl_c2", o["c2"])), tex,
                                           self._media_sdl(o))
        if t == abi.POV_OBJ_TORUS:
            return "torus { %s, %s %s%s }" % (_g(o["R"]), _g(o["r"]), o["mods"], tex)
        if t == abi.POV_OBJ_MESH:
            return self.meshes[o["mesh"]].sdl(self.materials[o["material"]])
        if t in (abi.POV_OBJ_UNION, abi.POV_OBJ_INTERSECTION, abi.POV_OBJ_MERGE):
            kids = " ".join(self._sdl_node(dict(c, inverted=False)) for c in o["children"])
            return "%s { %s translate %s%s }" % (o["kind"], kids, _v(o["translate"]), tex)
        raise ValueError("no SDL writer for object type %d" % t)

    # -- C ABI ---------------------------------------------------------------
    def camera(self):
        return camera_vectors(self.location, self.look_at, self.angle, self.right_len)

    def desc(self):
        """Returns (PovGpuSceneDesc, keepalive) -- keep the second alive while
        the first is in use."""
        keep = []
        flat = []

        def walk(o, parent):
            idx = len(flat)
            flat.append((o, parent))
            for c in o.get("children", ()):
                walk(c, idx)
            return idx

        for o in self.objects:
            walk(o, -1)
        n = len(flat)
        objs = (abi.PovGpuObject * max(n, 1))()
        first_child = {}
        for i, (o, parent) in enumerate(flat):
            if parent >= 0 and parent not in first_child:
                first_child[parent] = i
        for i, (o, parent) in enumerate(flat):
            d = objs[i]
            d.type = o["type"]
            d.flags = (abi.POV_FLAG_INVERTED if o.get("inverted") else 0) | \
                (abi.POV_FLAG_HOLLOW if o.get("hollow") else 0)
            d.media = int(o.get("media", 0))
            d.material = o.get("material", -1)
            d.parent = parent
            d.first_child = first_child.get(i, -1)
            d.num_children = len(o.get("children", ()))
            d.mesh = -1
            if o["type"] == abi.POV_OBJ_SPHERE:
                d.p[0], d.p[1], d.p[2] = o["centre"]
                d.p[3] = o["radius"]
            elif o["type"] == abi.POV_OBJ_PLANE:
                nrm = _normalized(o["normal"])
                d.p[0], d.p[1], d.p[2] = nrm
                d.p[3] = -o["offset"]
                d.flags |= abi.POV_FLAG_INFINITE
            elif o["type"] == abi.POV_OBJ_BOX:
                d.p[0], d.p[1], d.p[2] = o["c1"]
                d.p[3], d.p[4], d.p[5] = o["c2"]
            elif o["type"] == abi.POV_OBJ_TORUS:
                d.p[0], d.p[1] = o["R"], o["r"]
                d.flags |= abi.POV_FLAG_HAS_TRANS
                d.trans[:] = o["trans"].flat()
            elif o["type"] == abi.POV_OBJ_MESH:
                d.mesh = o["mesh"]
        mats = (abi.PovGpuMaterial * max(len(self.materials), 1))()
        pats, nrms = [], []
        for i, m in enumerate(self.materials):
            mats[i] = m.desc()
            if m.pattern is not None:
                pats.append(m.pattern.desc())
                mats[i].pattern = len(pats)
            if m.normal is not None:
                pats.append(m.normal.pattern.desc())
                nrms.append(m.normal.desc(len(pats)))
                mats[i].normal = len(nrms)
        lights = (abi.PovGpuLight * max(len(self.lights), 1))()
        for i, l in enumerate(self.lights):
            lights[i].center[:] = list(l["pos"])
            lights[i].colour[:] = list(l["rgb"])
            lights[i].kind = l["kind"]
            lights[i].adaptive_level = 100
            if l["kind"] == abi.POV_LIGHT_AREA:
                lights[i].axis1[:] = list(l["axis1"])
                lights[i].axis2[:] = list(l["axis2"])
                lights[i].area_size1, lights[i].area_size2 = l["size"]
                if l["adaptive"] is not None:
                    lights[i].adaptive_level = int(l["adaptive"])
                lights[i].circular = int(l["circular"])
                lights[i].orient = int(l["orient"])
            f = self._light_fields(l)
            lights[i].light_type = f["light_type"]
            lights[i].parallel = int(f["parallel"])
            lights[i].points_at[:] = list(f["points_at"])
            lights[i].radius, lights[i].falloff, lights[i].tightness = f["radius"], f["falloff"], f["tightness"]
            lights[i].fade_distance, lights[i].fade_power = f["fade_distance"], f["fade_power"]
        meshes = (abi.PovGpuMesh * max(len(self.meshes), 1))()
        for i, m in enumerate(self.meshes):
            meshes[i].vertices = m.vertices.ctypes.data_as(C.POINTER(C.c_float))
            meshes[i].num_vertices = len(m.vertices)
            if m.normals is not None:
                meshes[i].normals = m.normals.ctypes.data_as(C.POINTER(C.c_float))
                meshes[i].num_normals = len(m.normals)
                meshes[i].normal_indices = m.faces.ctypes.data_as(C.POINTER(C.c_int32))
            meshes[i].face_indices = m.faces.ctypes.data_as(C.POINTER(C.c_int32))
            meshes[i].num_triangles = m.num_triangles
            keep.append(m)
        desc = abi.PovGpuSceneDesc()
        desc.abi_version = abi.POV_GPU_ABI_VERSION
        desc.num_objects = n
        desc.objects = objs
        desc.num_materials = len(self.materials)
        desc.materials = mats
        desc.num_lights = len(self.lights)
        desc.lights = lights
        desc.num_meshes = len(self.meshes)
        desc.meshes = meshes
        dvec, rvec, uvec = self.camera()
        desc.camera.location[:] = list(self.location)
        desc.camera.direction[:] = list(dvec)
        desc.camera.right[:] = list(rvec)
        desc.camera.up[:] = list(uvec)
        desc.camera.type = 0
        desc.background[:] = [self.background[0], self.background[1], self.background[2], 0.0]
        desc.ambient_light[:] = [1.0, 1.0, 1.0]
        desc.max_trace_level = self.max_trace_level
        desc.adc_bailout = self.adc_bailout
        desc.language_version = 370
        desc.radiosity.enabled = 0
        medias = (abi.PovGpuMedia * max(len(self.medias), 1))()
        for i, md in enumerate(self.medias):
            m = medias[i]
            m.scattering_type = md["scattering_type"]
            m.eccentricity = md["eccentricity"] if md["scattering_type"] == 5 else 0.0
            m.method = 3
            m.intervals = md["intervals"]
            m.min_samples = m.max_samples = md["samples"]
            m.aa_level = md["aa_level"]
            m.aa_threshold = md["aa_threshold"]
            m.jitter = 0.0
            m.absorption[:] = list(md["absorption"])
            m.emission[:] = list(md["emission"])
            m.scattering[:] = list(md["scattering"])
            m.extinction[:] = [a + sc for a, sc in zip(md["absorption"], md["scattering"])]
        desc.num_medias = len(self.medias)
        desc.medias = medias
        keep.append(medias)
        patterns = (abi.PovGpuPattern * max(len(pats), 1))(*pats)
        desc.num_patterns = len(pats)
        desc.patterns = patterns
        keep.append(patterns)
        normals = (abi.PovGpuNormal * max(len(nrms), 1))(*nrms)
        desc.num_normals = len(nrms)
        desc.normals = normals
        keep.append(normals)
        # interiors: every object has one (Parser::Post_Process gives an
        # object without interior{} a default one, parser.cpp:9225-9230, and
        # a CSG child without its own its parent's, parser.cpp:9040-9044)
        ints, obj_int = [], (C.c_int32 * max(n, 1))()
        for i, (o, parent) in enumerate(flat):
            if o.get("interior") is not None:
                ints.append(o["interior"].desc())
                obj_int[i] = len(ints)
            elif parent >= 0:
                obj_int[i] = obj_int[parent]
            else:
                ints.append(Interior().desc())
                obj_int[i] = len(ints)
        interiors = (abi.PovGpuInterior * max(len(ints), 1))(*ints)
        desc.num_interiors = len(ints)
        desc.interiors = interiors
        desc.object_interior = obj_int
        desc.atmosphere_ior = 1.0
        keep += [interiors, obj_int]
        if self.radiosity is not None:
            r = self.radiosity_settings()
            rd = desc.radiosity
            rd.enabled = 1
            rd.count, rd.recursion_limit, rd.nearest_count = r["count"], r["recursion_limit"], r["nearest_count"]
            rd.error_bound, rd.low_error_factor, rd.gray_threshold = r["error_bound"], r["low_error_factor"], \
                r["gray_threshold"]
            rd.minimum_reuse, rd.maximum_reuse, rd.brightness = r["minimum_reuse"], r["maximum_reuse"], \
                r["brightness"]
            rd.pretrace_start, rd.pretrace_end, rd.adc_bailout = r["pretrace_start"], r["pretrace_end"], \
                r["adc_bailout"]
            rd.always_sample = int(r["always_sample"])
        keep += [objs, mats, lights, meshes]
        return desc, keep

    def render_params(self):
        p = abi.PovGpuRenderParams()
        p.width = self.width
        p.height = self.height
        if self.antialias is not None:
            p.antialias = 1
            p.sampling_method = 2
            p.aa_threshold, p.aa_depth = self.antialias
        else:
            p.antialias = 0
            p.sampling_method = 1
        p.quality = 9
        return p

    def camera_rays(self, xs=None, ys=None):
        """Primary rays through pixel centres (x+0.5, y+0.5) exactly as
        TracePixel::CreateCameraRay forms them
        (source/core/render/tracepixel.cpp:357-373,924), in float64."""
        dvec, rvec, uvec = (np.array(v) for v in self.camera())
        if xs is None:
            yy, xx = np.mgrid[0:self.height, 0:self.width]
            xs, ys = xx.ravel(), yy.ravel()
        x0 = (np.asarray(xs, dtype=np.float64) + 0.5) / self.width - 0.5
        y0 = 0.5 - (np.asarray(ys, dtype=np.float64) + 0.5) / self.height
        d = dvec[None, :] + x0[:, None] * rvec[None, :] + y0[:, None] * uvec[None, :]
        d = d / np.sqrt((d * d).sum(axis=1))[:, None]
        o = np.broadcast_to(np.array(self.location), d.shape).copy()
        return np.ascontiguousarray(o), np.ascontiguousarray(d)


def blocks_for(width, height, block=32):
    """The view's render-block grid (source/backend/scene/view.cpp:810-822)."""
    out = []
    serial = 0
    for top in range(0, height, block):
        for left in range(0, width, block):
            out.append((left, top, min(left + block, width) - 1, min(top + block, height) - 1, serial))
            serial += 1
    return out


class BlockBatch:
    """Render blocks packed once for the C ABI: the PovGpuBlock array
    (`arr`, over a numpy buffer), the block list and the pixels it covers.
    The render calls take one in place of a list, so a caller that traces
    the same blocks every frame packs them once (the reference's render
    task hands the library its C array the same way)."""

    def __init__(self, blocks):
        self.blocks = list(blocks)
        buf = np.zeros((len(self.blocks), 6), dtype=np.int32)   # left, top, right, bottom, serial, reserved
        if self.blocks:
            buf[:, :5] = np.asarray(self.blocks, dtype=np.int64)
        self._buf = buf
        self.arr = (abi.PovGpuBlock * len(self.blocks)).from_buffer(buf)
        w = buf[:, 2].astype(np.int64) - buf[:, 0] + 1
        h = buf[:, 3].astype(np.int64) - buf[:, 1] + 1
        self.npix = int((w * h).sum())

    def __len__(self):
        return len(self.blocks)

    def __iter__(self):
        return iter(self.blocks)


def block_batch(blocks):
    return blocks if isinstance(blocks, BlockBatch) else BlockBatch(blocks)


def block_array(blocks):
    return block_batch(blocks).arr


def unblock(rgbt, blocks, width, height):
    """Scatters block-ordered RGBT back into an image (H, W, 4)."""
    img = np.zeros((height, width, 4), dtype=np.float32)
    off = 0
    for (l, t, r, b, _s) in blocks:
        w, h = r - l + 1, b - t + 1
        img[t:b + 1, l:r + 1] = rgbt[off:off + w * h].reshape(h, w, 4)
        off += w * h
    return img


# -------------------------------------------------------------- generators --
def spheres_plane(width=320, height=240, n_spheres=64, seed=1):
    """64 spheres, centres U[-10,10]^3, radii U[0.2,1.0], rgb U[0,1]^3 (seed 1);
    plane y=-10; point lights (20,30,-20), (-15,25,-10); phong 0.5;
    max_trace_level 1; camera (0,5,-25) looking at the origin, 50 deg."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-10.0, 10.0, size=(n_spheres, 3))
    radii = rng.uniform(0.2, 1.0, size=n_spheres)
    colours = rng.uniform(0.0, 1.0, size=(n_spheres, 3))
    s = Scene("spheres_plane", width, height, (0.0, 5.0, -25.0), (0.0, 0.0, 0.0), 50.0,
              max_trace_level=1)
    s.point_light((20.0, 30.0, -20.0))
    s.point_light((-15.0, 25.0, -10.0))
    for i in range(n_spheres):
        m = s.material(Material(colours[i], phong=0.5))
        s.sphere(centres[i], radii[i], m)
    s.plane((0.0, 1.0, 0.0), -10.0, s.material(Material((0.8, 0.8, 0.8), phong=0.5)))
    return s


def _value_noise3(p, seed, octaves=3):
    """Sum of `octaves` octaves of trilinear value noise on an integer lattice
    with smoothstep weights; lattice values are a hash of (i, j, k, seed)
    mapped to [-1, 1]."""
    total = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 2.0, 0.0
    for o in range(octaves):
        q = p * freq + 17.0 * (o + 1)
        i0 = np.floor(q).astype(np.int64)
        f = q - i0
        w = f * f * (3.0 - 2.0 * f)

        def lattice(di, dj, dk):
            h = ((i0[:, 0] + di) * 73856093) ^ ((i0[:, 1] + dj) * 19349663) ^ \
                ((i0[:, 2] + dk) * 83492791) ^ (seed * 2654435761 + o * 97)
            h = (h ^ (h >> 13)) * 1274126177
            h = h ^ (h >> 16)
            return (h & 0xFFFF).astype(np.float64) / 32767.5 - 1.0

        acc = 0.0
        for di in (0, 1):
            for dj in (0, 1):
                for dk in (0, 1):
                    wx = w[:, 0] if di else 1.0 - w[:, 0]
                    wy = w[:, 1] if dj else 1.0 - w[:, 1]
                    wz = w[:, 2] if dk else 1.0 - w[:, 2]
                    acc = acc + wx * wy * wz * lattice(di, dj, dk)
        total += amp * acc
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def displaced_sphere_mesh(n=296, amplitude=0.15, radius=8.0, seed=2):
    """Cube-sphere with n x n quads per face (6*n*n*2 triangles; n=296 gives
    1,051,392), every vertex pushed radially by 3-octave value noise of
    amplitude `amplitude`, scaled to `radius`, with per-vertex normals
    averaged from the adjacent faces (area weighted)."""
    verts, faces = [], []
    base = 0
    g = np.linspace(-1.0, 1.0, n + 1)
    uu, vv = np.meshgrid(g, g, indexing="ij")
    axes = [(0, 1, 2, 1.0), (0, 1, 2, -1.0), (1, 2, 0, 1.0), (1, 2, 0, -1.0),
            (2, 0, 1, 1.0), (2, 0, 1, -1.0)]
    idx = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    for (a, b, c, sgn) in axes:
        p = np.zeros(((n + 1) * (n + 1), 3))
        p[:, a] = uu.ravel()
        p[:, b] = vv.ravel() * sgn
        p[:, c] = sgn
        verts.append(p)
        q00 = idx[:-1, :-1].ravel() + base
        q10 = idx[1:, :-1].ravel() + base
        q01 = idx[:-1, 1:].ravel() + base
        q11 = idx[1:, 1:].ravel() + base
        faces.append(np.stack([q00, q10, q11], axis=1))
        faces.append(np.stack([q00, q11, q01], axis=1))
        base += (n + 1) * (n + 1)
    p = np.concatenate(verts)
    f = np.concatenate(faces).astype(np.int32)
    d = p / np.linalg.norm(p, axis=1)[:, None]
    r = 1.0 + amplitude * _value_noise3(d, seed)
    pos = (d * (r * radius)[:, None]).astype(np.float32)
    v0, v1, v2 = (pos[f[:, k]].astype(np.float64) for k in range(3))
    fn = np.cross(v1 - v0, v2 - v0)
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    # make seam duplicates share one normal: accumulate by position
    key = np.round(pos.astype(np.float64) * 1e5).astype(np.int64)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    inv = inv.ravel()
    acc = np.zeros((inv.max() + 1, 3))
    np.add.at(acc, inv, vn)
    vn = acc[inv]
    vn /= np.linalg.norm(vn, axis=1)[:, None]
    return Mesh(pos, vn.astype(np.float32), f)


def mesh_spheres(width=1920, height=1080, mesh_n=296, n_spheres=1024, seed=2):
    """The 1M-triangle scene: displaced sphere mesh2 (radius 8) + 1024 spheres
    r U[0.1,0.5] in [-12,12]^3 + plane y=-9; one point light with shadows;
    reflection 0.3 on every surface; max_trace_level 3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-12.0, 12.0, size=(n_spheres, 3))
    radii = rng.uniform(0.1, 0.5, size=n_spheres)
    colours = rng.uniform(0.0, 1.0, size=(n_spheres, 3))
    s = Scene("mesh_spheres", width, height, (0.0, 5.0, -25.0), (0.0, 0.0, 0.0), 50.0,
              max_trace_level=3)
    s.point_light((20.0, 30.0, -20.0))
    mesh = displaced_sphere_mesh(n=mesh_n, seed=seed)
    s.mesh(mesh, s.material(Material((0.9, 0.7, 0.4), phong=0.5, reflection=0.3)))
    for i in range(n_spheres):
        s.sphere(centres[i], radii[i], s.material(Material(colours[i], phong=0.5, reflection=0.3)))
    s.plane((0.0, 1.0, 0.0), -9.0, s.material(Material((0.8, 0.8, 0.8), phong=0.5, reflection=0.3)))
    return s


def csg_torus_grid(width=1920, height=1080, n=16, seed=3, antialias=(0.1, 3)):
    """CSG and quartic batch: n^3 objects on a grid of spacing 2 centred on the
    origin, each jittered by U[-0.3,0.3]^3 (seed 3), cycling through
      difference(box +-0.6, sphere r0.7), intersection(sphere r0.8, box +-0.5),
      merge(two spheres r0.5, centres 0.4 apart), torus(0.6, 0.15) with a
      random rotation;
    random rgb pigments, 2 shadowing point lights, reflection 0.2,
    max_trace_level 4, adaptive antialiasing (method 2) threshold 0.1 depth 3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    count = n ** 3
    jit = rng.uniform(-0.3, 0.3, size=(count, 3))
    rot = rng.uniform(0.0, 360.0, size=(count, 3))
    col = rng.uniform(0.0, 1.0, size=(count, 3))
    s = Scene("csg_torus_grid", width, height, (0.0, 18.0, -42.0), (0.0, 0.0, 0.0), 50.0, max_trace_level=4)
    s.point_light((30.0, 40.0, -30.0))
    s.point_light((-30.0, 30.0, -20.0))
    s.antialias = antialias
    k = 0
    for i in range(n):
        for j in range(n):
            for l in range(n):
                c = ((i - (n - 1) / 2.0) * 2.0 + jit[k, 0], (j - (n - 1) / 2.0) * 2.0 + jit[k, 1],
                     (l - (n - 1) / 2.0) * 2.0 + jit[k, 2])
                m = s.material(Material(col[k], phong=0.5, reflection=0.2))
                kind = k % 4
                if kind == 0:
                    node = Scene.n_csg("difference", [Scene.n_box((-0.6, -0.6, -0.6), (0.6, 0.6, 0.6)),
                                                      Scene.n_sphere((0.0, 0.0, 0.0), 0.7)], c, m)
                elif kind == 1:
                    node = Scene.n_csg("intersection", [Scene.n_sphere((0.0, 0.0, 0.0), 0.8),
                                                        Scene.n_box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))], c, m)
                elif kind == 2:
                    node = Scene.n_csg("merge", [Scene.n_sphere((-0.2, 0.0, 0.0), 0.5),
                                                 Scene.n_sphere((0.2, 0.0, 0.0), 0.5)], c, m)
                else:
                    node = Scene.n_torus(0.6, 0.15, rot[k], c, m)
                s.add(node)
                k += 1
    return s


def torus_tunnel(width=160, height=120, n_rings=48, csg_child=False):
    """A tunnel of `n_rings` tori (major 3, minor 0.3, rings facing the
    camera, every 2 units along +z from z=2) ending at a wall (plane z=100),
    seen from (0,0,-5) looking down the axis, one light beside the camera:
    every camera ray passes a few dozen tori, so the traversal's list of
    deferred torus tests fills up and the rays beyond it take the second,
    ordinary traversal.  With `csg_child` the last ring is a torus merged
    with a sphere (a CSG with a torus child: no torus-free variant).  Reflection 0.3 on the rings, max_trace_level 3."""
    s = Scene("torus_tunnel", width, height, (0.0, 0.0, -5.0), (0.0, 0.0, 100.0), 60.0, max_trace_level=3)
    s.point_light((1.0, 1.5, -4.0))
    wall = s.material(Material((0.8, 0.8, 0.7)))
    s.plane((0.0, 0.0, -1.0), -100.0, wall)
    rng = np.random.Generator(np.random.PCG64(9))
    for k in range(n_rings):
        m = s.material(Material(tuple(rng.uniform(0.2, 1.0, 3)), phong=0.4, reflection=0.3))
        node = Scene.n_torus(3.0, 0.3, (90.0, 0.0, 0.0), (0.0, 0.0, 2.0 + 2.0 * k), m)
        if csg_child and k == n_rings - 1:
            node = Scene.n_csg("merge", [node, Scene.n_sphere((0.0, 0.0, 2.0 + 2.0 * k), 0.5)], mat=m)
        s.add(node)
    return s


def radiosity_room(width=1280, height=720, n_spheres=200, seed=4, radiosity=True, count=200,
                   recursion_limit=2, error_bound=0.5, area=(4, 4), adaptive=None, circular=False,
                   orient=False):
    """Box room [-10,10]^3 as six planes, diffuse 0.7 walls (x=-10 rgb
    <0.7,0.1,0.1>, x=+10 rgb <0.1,0.7,0.1>, the others rgb 0.9);
    `n_spheres` spheres r U[0.3,1.5], centres x,z U[-8.5,8.5], y U[-8.5,4]
    (the space under the light kept clear), rgb U[0.2,0.9]^3 (seed 4), none
    within 6 of the camera; ceiling area light at (0,9,0),
    area_light <2,0,0>,<0,0,2>,4,4; ambient 0 everywhere;
    radiosity { count 200 recursion_limit 2 error_bound 0.5 } when
    `radiosity`; camera (0,4,-9.5) looking at (0,-3,0), 75 deg."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("radiosity_room", width, height, (0.0, 4.0, -9.5), (0.0, -3.0, 0.0), 75.0,
              max_trace_level=3)
    s.area_light((0.0, 9.0, 0.0), (2.0, 0.0, 0.0), (0.0, 0.0, 2.0), area[0], area[1], adaptive=adaptive,
                 circular=circular, orient=orient)
    white = s.material(Material((0.9, 0.9, 0.9), ambient=0.0, diffuse=0.7))
    red = s.material(Material((0.7, 0.1, 0.1), ambient=0.0, diffuse=0.7))
    green = s.material(Material((0.1, 0.7, 0.1), ambient=0.0, diffuse=0.7))
    s.plane((0.0, 1.0, 0.0), -10.0, white)     # floor
    s.plane((0.0, -1.0, 0.0), -10.0, white)    # ceiling
    s.plane((1.0, 0.0, 0.0), -10.0, red)       # x = -10
    s.plane((-1.0, 0.0, 0.0), -10.0, green)    # x = +10
    s.plane((0.0, 0.0, 1.0), -10.0, white)     # z = -10
    s.plane((0.0, 0.0, -1.0), -10.0, white)    # z = +10
    cam = np.array(s.location)
    placed = 0
    while placed < n_spheres:
        c = np.array([rng.uniform(-8.5, 8.5), rng.uniform(-8.5, 4.0), rng.uniform(-8.5, 8.5)])
        r = rng.uniform(0.3, 1.5)
        rgb = rng.uniform(0.2, 0.9, size=3)
        if np.linalg.norm(c - cam) < r + 6.0:
            continue
        s.sphere(c, r, s.material(Material(rgb, ambient=0.0, diffuse=0.7)))
        placed += 1
    if radiosity:
        s.radiosity = dict(count=count, recursion_limit=recursion_limit, error_bound=error_bound)
    return s


def media_spheres(width=320, height=240, n_spheres=24, seed=5, intervals=10, samples=10, scattering=0.05,
                  scattering_type=1, eccentricity=0.0, absorption=(0.0, 0.0, 0.0), emission=(0.0, 0.0, 0.0),
                  container="box"):
    """A uniform scattering media box [-7,7]^3 (hollow, fully transmitting;
    scattering {1, rgb 0.05} -- or another scattering type, with its
    eccentricity for Henyey-Greenstein, absorption and emission; with
    container="sphere" a hollow sphere of radius 11 at the origin holds it --,
    intervals 10, samples 10, method 3) around
    `n_spheres` spheres r U[0.4,1.2], centres U[-5.5,5.5]^3, rgb U[0.2,0.9]^3
    (seed 5), every other one with reflection 0.2; plane y=-8; one point
    light (20,30,-20); camera (0,4,-25) looking at the origin, 50 deg;
    max_trace_level 3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("media_spheres", width, height, (0.0, 4.0, -25.0), (0.0, 0.0, 0.0), 50.0, max_trace_level=3)
    s.point_light((20.0, 30.0, -20.0))
    s.media_box((-7.0, -7.0, -7.0), (7.0, 7.0, 7.0), scattering=(scattering,) * 3, intervals=intervals,
                samples=samples, scattering_type=scattering_type, eccentricity=eccentricity, absorption=absorption,
                emission=emission, sphere=((0.0, 0.0, 0.0), 11.0) if container == "sphere" else None)
    for i in range(n_spheres):
        c = rng.uniform(-5.5, 5.5, size=3)
        r = rng.uniform(0.4, 1.2)
        rgb = rng.uniform(0.2, 0.9, size=3)
        s.sphere(c, r, s.material(Material(rgb, phong=0.4, reflection=0.2 if i % 2 else 0.0)))
    s.plane((0.0, 1.0, 0.0), -8.0, s.material(Material((0.8, 0.8, 0.8))))
    return s


def textured_spheres(width=320, height=240, n_spheres=12, seed=6, noise_generator=None, turbulent=False):
    """Pattern pigments: a checker floor (plane y=-2, checker scale 1.5),
    `n_spheres` spheres r U[0.5,1.2] in a 6x6 area (seed 6) cycling through
    bozo (3-entry colour map, scale 0.4), granite (scale 1.5), gradient y
    (scale 2, translated) and bozo rotated -- or, with `turbulent`, marble
    and wood with turbulence, agate, onion, leopard, bozo with turbulence
    (3 octaves), a sine-wave gradient with frequency and phase and granite
    with turbulence; one point light, phong 0.3; camera (0,3,-10) looking
    at (0,0,2), 55 deg; max_trace_level 2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("textured_spheres", width, height, (0.0, 3.0, -10.0), (0.0, 0.0, 2.0), 55.0, max_trace_level=2)
    s.point_light((10.0, 15.0, -10.0))
    ng = noise_generator
    floor = Pattern("checker", [(0.0, (0.9, 0.9, 0.9)), (1.0, (0.15, 0.2, 0.5))], [("scale", (1.5, 1.5, 1.5))])
    s.plane((0.0, 1.0, 0.0), -2.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    kinds = [
        Pattern("bozo", [(0.0, (0.9, 0.3, 0.1)), (0.5, (0.95, 0.9, 0.3)), (1.0, (0.1, 0.5, 0.2))],
                [("scale", (0.4, 0.4, 0.4))], noise_generator=ng),
        Pattern("granite", [(0.0, (0.2, 0.2, 0.25)), (0.4, (0.8, 0.7, 0.7)), (1.0, (0.95, 0.95, 0.9))],
                [("scale", (1.5, 1.5, 1.5))], noise_generator=ng),
        Pattern("gradient", [(0.0, (0.1, 0.2, 0.8)), (1.0, (0.9, 0.9, 1.0))],
                [("scale", (2.0, 2.0, 2.0)), ("translate", (0.0, 0.3, 0.0))], gradient=(0.0, 1.0, 0.0)),
        Pattern("bozo", [(0.0, (0.1, 0.1, 0.1)), (0.3, (0.6, 0.2, 0.6)), (1.0, (1.0, 1.0, 1.0))],
                [("scale", (0.7, 0.3, 0.7)), ("rotate", (20.0, 35.0, 0.0))], noise_generator=ng),
    ]
    if turbulent:
        warm = [(0.0, (0.9, 0.85, 0.7)), (0.6, (0.6, 0.3, 0.15)), (1.0, (0.2, 0.1, 0.05))]
        cool = [(0.0, (0.05, 0.1, 0.3)), (0.5, (0.5, 0.7, 0.9)), (1.0, (1.0, 1.0, 1.0))]
        kinds = [
            Pattern("marble", cool, [("scale", (0.8, 0.8, 0.8))], turbulence=(0.7, 0.7, 0.7), noise_generator=ng),
            Pattern("wood", warm, [("scale", (0.15, 0.15, 0.15)), ("rotate", (90.0, 0.0, 0.0))],
                    turbulence=(0.05, 0.05, 0.05)),
            Pattern("agate", warm, [("scale", (0.5, 0.5, 0.5))], agate_turb=0.8, noise_generator=ng),
            Pattern("onion", cool, [("scale", (0.3, 0.3, 0.3))]),
            Pattern("leopard", warm, [("scale", (0.1, 0.1, 0.1))]),
            Pattern("bozo", cool, [("scale", (0.5, 0.5, 0.5))], turbulence=(0.5, 0.3, 0.5), octaves=3, omega=0.6,
                    lambda_=2.5, noise_generator=ng),
            Pattern("gradient", warm, gradient=(1.0, 1.0, 0.0), wave="sine", frequency=2.0, phase=0.25),
            Pattern("granite", cool, [("scale", (2.0, 2.0, 2.0))], turbulence=(0.3, 0.3, 0.3), noise_generator=ng),
        ]
    for i in range(n_spheres):
        c = (rng.uniform(-3.0, 3.0), rng.uniform(-1.0, 1.5), rng.uniform(0.0, 6.0))
        r = rng.uniform(0.5, 1.2)
        s.sphere(c, r, s.material(Material((1.0, 1.0, 1.0), phong=0.3, pattern=kinds[i % len(kinds)])))
    return s


def light_types(width=320, height=240, seed=7):
    """The light source kinds on one floor: 14 spheres r U[0.5,1.1] on a
    ring of radius 5.5 (seed 7, rgb U[0.3,1], phong 0.6) over the plane y=0
    (grey 0.8, phong 0.3, reflection 0.1), camera (0,7,-17) looking at
    (0,0.5,0), 50 degrees, max_trace_level 3.  Lights: a spotlight at
    (-6,12,-4) on (-2,0,0), radius 15, falloff 25, tightness 5, fade_distance
    12, fade_power 2; a cylinder light at (8,10,4) on (3,0,2), radius 1.5,
    falloff 3, tightness 1; a parallel light at (0,20,-20) on the origin; a
    shadowless fill light at (0,10,-15); a 3x3 area spotlight at (5,9,-6)
    (axes <1.5,0,0>, <0,0,1.5>, adaptive 1) on (2,0,0), radius 20, falloff
    30."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 14
    ang = np.arange(n) * (2.0 * math.pi / n) + rng.uniform(-0.1, 0.1, size=n)
    radii = rng.uniform(0.5, 1.1, size=n)
    colours = rng.uniform(0.3, 1.0, size=(n, 3))
    s = Scene("light_types", width, height, (0.0, 7.0, -17.0), (0.0, 0.5, 0.0), 50.0, max_trace_level=3)
    s.light((-6.0, 12.0, -4.0), (1.5, 1.35, 1.05), beam="spotlight", radius=15.0, falloff=25.0, tightness=5.0,
            point_at=(-2.0, 0.0, 0.0), fade_distance=12.0, fade_power=2.0)
    s.light((8.0, 10.0, 4.0), (0.5, 0.7, 1.0), beam="cylinder", radius=1.5, falloff=3.0, tightness=1.0,
            point_at=(3.0, 0.0, 2.0))
    s.light((0.0, 20.0, -20.0), (0.3, 0.3, 0.3), point_at=(0.0, 0.0, 0.0), parallel=True)
    s.light((0.0, 10.0, -15.0), (0.15, 0.15, 0.15), shadowless=True)
    s.area_light((5.0, 9.0, -6.0), (1.5, 0.0, 0.0), (0.0, 0.0, 1.5), 3, 3, rgb=(0.6, 0.4, 0.4), adaptive=1)
    s.lights[-1].update(beam="spotlight", radius=20.0, falloff=30.0, point_at=(2.0, 0.0, 0.0))
    for i in range(n):
        c = (5.5 * math.cos(ang[i]), radii[i], 5.5 * math.sin(ang[i]))
        s.sphere(c, radii[i], s.material(Material(colours[i], phong=0.6)))
    s.plane((0.0, 1.0, 0.0), 0.0, s.material(Material((0.8, 0.8, 0.8), phong=0.3, reflection=0.1)))
    return s


def glass_spheres(width=320, height=240, max_trace_level=10):
    """Refraction and interiors: over a checker floor (plane y=-1) and a
    checker wall (z=9), transparent spheres -- clear glass (rgb 1, filter
    0.9, ior 1.5), tinted glass (rgb <1,0.45,0.45>, filter 0.85, ior 1.33),
    a transmit-only ball (transmit 0.7, ior 1: transmitted rays), dense glass
    (ior 2.4: total internal reflection towards its rim), a fading sphere
    (fade_distance 1.2, fade_power 2, fade colour <0.4,0.7,1>), an
    exponential fade (fade_power 1001), a big glass sphere holding a small
    one of another ior, two overlapping glass spheres, a glass CSG
    intersection of a sphere and a box (one interior) -- in front of three
    opaque spheres; two point lights whose shadows pass through the glass.
    Transparent surfaces have phong highlights but no reflection.  Camera
    (0,3,-12) looking at (0,0.5,0), 55 deg; max_trace_level 10."""
    s = Scene("glass_spheres", width, height, (0.0, 3.0, -12.0), (0.0, 0.5, 0.0), 55.0,
              max_trace_level=max_trace_level)
    s.point_light((8.0, 14.0, -10.0))
    s.point_light((-10.0, 9.0, -4.0), (0.5, 0.5, 0.55))
    # the checkers are shifted half a square across their planes: a plane
    # lying on a checker boundary takes its colour from the rounding of
    # the hit point, which FP32 and FP64 round differently
    floor = Pattern("checker", [(0.0, (0.9, 0.9, 0.85)), (1.0, (0.2, 0.3, 0.55))],
                    [("scale", (1.0, 1.0, 1.0)), ("translate", (0.0, 0.5, 0.0))])
    wall = Pattern("checker", [(0.0, (0.85, 0.6, 0.3)), (1.0, (0.95, 0.95, 0.9))],
                   [("scale", (1.5, 1.5, 1.5)), ("translate", (0.0, 0.0, 0.75))])
    s.plane((0.0, 1.0, 0.0), -1.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    s.plane((0.0, 0.0, -1.0), -9.0, s.material(Material((1.0, 1.0, 1.0), pattern=wall)))
    for c, r, rgb in (((-3.0, 0.2, 5.0), 1.2, (0.8, 0.2, 0.15)), ((1.5, 0.0, 6.0), 1.0, (0.2, 0.7, 0.25)),
                      ((4.5, 0.5, 4.0), 1.5, (0.25, 0.3, 0.85))):
        s.sphere(c, r, s.material(Material(rgb, phong=0.4)))

    def glass(rgb=(1.0, 1.0, 1.0), filter=0.0, transmit=0.0):
        return s.material(Material(rgb, ambient=0.0, diffuse=0.1, phong=0.8, phong_size=80.0, filter=filter,
                                   transmit=transmit))
    s.sphere((-4.2, 0.0, 0.0), 1.0, glass(filter=0.9), Interior(ior=1.5))
    s.sphere((-1.8, 0.0, -0.5), 1.0, glass((1.0, 0.45, 0.45), filter=0.85), Interior(ior=1.33))
    s.sphere((0.6, 0.0, 0.0), 1.0, glass((0.6, 0.9, 0.6), transmit=0.7), Interior(ior=1.0))
    s.sphere((3.0, 0.0, -0.5), 1.0, glass(filter=0.95), Interior(ior=2.4))
    s.sphere((-3.0, 2.6, 1.5), 0.9, glass(filter=0.9),
             Interior(ior=1.45, fade_distance=1.2, fade_power=2.0, fade_colour=(0.4, 0.7, 1.0)))
    s.sphere((-0.6, 2.7, 1.8), 0.9, glass(filter=0.9),
             Interior(ior=1.2, fade_distance=0.8, fade_power=1001.0, fade_colour=(1.0, 0.6, 0.3)))
    s.sphere((2.4, 2.8, 2.0), 1.3, glass(filter=0.92), Interior(ior=1.5))          # holds the next one
    s.sphere((2.4, 2.8, 2.0), 0.5, glass((0.5, 0.6, 1.0), filter=0.8), Interior(ior=1.9))
    s.sphere((-5.0, 2.4, 3.5), 0.8, glass(filter=0.9), Interior(ior=1.3))             # two overlapping
    s.sphere((-4.3, 2.6, 3.3), 0.7, glass((1.0, 1.0, 0.6), filter=0.9), Interior(ior=1.6))
    s.add(Scene.n_csg("intersection", [Scene.n_sphere((0.0, 0.0, 0.0), 0.9),
                                       Scene.n_box((-0.65, -0.65, -0.65), (0.65, 0.65, 0.65))],
                      translate=(5.3, 0.0, 1.0), mat=glass((0.7, 0.8, 1.0), filter=0.9), interior=Interior(ior=1.5)))
    return s


def glass_reflective(width=320, height=240, max_trace_level=8):
    """Transparent surfaces that also reflect, so a hit traces the refracted
    ray and then the reflected one: over the checker floor and wall of
    glass_spheres, glass with fresnel reflection and conserve_energy
    (reflection { 0, 1 fresnel on }, filter 0.9, ior 1.5), the same tinted
    (rgb <1,0.6,0.4>, ior 1.33), dense fresnel glass (ior 2.4: total
    internal reflection skips the reflection), glass with a constant
    reflection 0.1 (filter 0.9, ior 1.5), a transmit-only ball with
    reflection 0.15 (ior 1: transmitted rays), a fresnel glass sphere
    holding an opaque mirror ball (reflection 0.6: its reflected rays keep
    the glass's interior), two overlapping fresnel spheres of other iors,
    and three opaque spheres with reflection 0.3 behind; two point lights.
    Camera (0,3,-12) looking at (0,0.5,0), 55 deg; max_trace_level 8."""
    s = Scene("glass_reflective", width, height, (0.0, 3.0, -12.0), (0.0, 0.5, 0.0), 55.0,
              max_trace_level=max_trace_level)
    s.point_light((8.0, 14.0, -10.0))
    s.point_light((-10.0, 9.0, -4.0), (0.5, 0.5, 0.55))
    floor = Pattern("checker", [(0.0, (0.9, 0.9, 0.85)), (1.0, (0.2, 0.3, 0.55))],
                    [("scale", (1.0, 1.0, 1.0)), ("translate", (0.0, 0.5, 0.0))])
    wall = Pattern("checker", [(0.0, (0.85, 0.6, 0.3)), (1.0, (0.95, 0.95, 0.9))],
                   [("scale", (1.5, 1.5, 1.5)), ("translate", (0.0, 0.0, 0.75))])
    s.plane((0.0, 1.0, 0.0), -1.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    s.plane((0.0, 0.0, -1.0), -9.0, s.material(Material((1.0, 1.0, 1.0), pattern=wall)))
    for c, r, rgb in (((-3.0, 0.2, 5.0), 1.2, (0.8, 0.2, 0.15)), ((1.5, 0.0, 6.0), 1.0, (0.2, 0.7, 0.25)),
                      ((4.5, 0.5, 4.0), 1.5, (0.25, 0.3, 0.85))):
        s.sphere(c, r, s.material(Material(rgb, phong=0.4, reflection=0.3)))

    def glass(rgb=(1.0, 1.0, 1.0), filter=0.0, transmit=0.0, fresnel=True, reflection=1.0):
        return s.material(Material(rgb, ambient=0.0, diffuse=0.1, phong=0.8, phong_size=80.0, filter=filter,
                                   transmit=transmit, reflection=reflection,
                                   reflection_min=0.0 if fresnel else None, fresnel=fresnel,
                                   conserve_energy=fresnel))
    s.sphere((-4.2, 0.0, 0.0), 1.0, glass(filter=0.9), Interior(ior=1.5))
    s.sphere((-1.8, 0.0, -0.5), 1.0, glass((1.0, 0.6, 0.4), filter=0.85), Interior(ior=1.33))
    s.sphere((0.6, 0.0, 0.0), 1.0, glass((0.6, 0.9, 0.6), transmit=0.7, fresnel=False, reflection=0.15),
             Interior(ior=1.0))
    s.sphere((3.0, 0.0, -0.5), 1.0, glass(filter=0.95), Interior(ior=2.4))
    s.sphere((-3.0, 2.6, 1.5), 0.9, glass(filter=0.9, fresnel=False, reflection=0.1), Interior(ior=1.5))
    s.sphere((2.4, 2.8, 2.0), 1.3, glass(filter=0.92), Interior(ior=1.5))          # holds the mirror ball
    s.sphere((2.4, 2.8, 2.0), 0.45, s.material(Material((0.9, 0.9, 0.9), phong=0.6, reflection=0.6)))
    s.sphere((-0.6, 2.5, 2.5), 0.9, glass(filter=0.9), Interior(ior=1.3))             # two overlapping
    s.sphere((0.1, 2.7, 2.3), 0.7, glass((1.0, 1.0, 0.6), filter=0.9), Interior(ior=1.6))
    return s


def glass_patterns(width=320, height=240, max_trace_level=8):
    """Pattern pigments whose colour maps filter or transmit, so a surface
    is transparent where the blended colour is: over the checker floor and
    wall of glass_spheres, a sphere of checker squares alternately clear
    glass (filter 0.9) and opaque red, a marble sphere with filtering
    veins, a gradient sphere from opaque blue to transmit 0.8, a bozo
    sphere of clouded glass (ior 1.4), a crackle ball whose cells transmit,
    and a glass box with an onion map (ior 1.3); opaque spheres behind;
    two point lights whose shadows pass through the patterns.  Camera
    (0,3,-12) looking at (0,0.5,0), 55 deg; max_trace_level 8."""
    s = Scene("glass_patterns", width, height, (0.0, 3.0, -12.0), (0.0, 0.5, 0.0), 55.0,
              max_trace_level=max_trace_level)
    s.point_light((8.0, 14.0, -10.0))
    s.point_light((-10.0, 9.0, -4.0), (0.5, 0.5, 0.55))
    floor = Pattern("checker", [(0.0, (0.9, 0.9, 0.85)), (1.0, (0.2, 0.3, 0.55))],
                    [("scale", (1.0, 1.0, 1.0)), ("translate", (0.0, 0.5, 0.0))])
    wall = Pattern("checker", [(0.0, (0.85, 0.6, 0.3)), (1.0, (0.95, 0.95, 0.9))],
                   [("scale", (1.5, 1.5, 1.5)), ("translate", (0.0, 0.0, 0.75))])
    s.plane((0.0, 1.0, 0.0), -1.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    s.plane((0.0, 0.0, -1.0), -9.0, s.material(Material((1.0, 1.0, 1.0), pattern=wall)))
    for c, r, rgb in (((-3.0, 0.2, 5.0), 1.2, (0.8, 0.2, 0.15)), ((1.5, 0.0, 6.0), 1.0, (0.2, 0.7, 0.25)),
                      ((4.5, 0.5, 4.0), 1.5, (0.25, 0.3, 0.85))):
        s.sphere(c, r, s.material(Material(rgb, phong=0.4)))
    off = ("translate", (0.131, 0.077, 0.219))

    def glass(pattern):
        return s.material(Material((1.0, 1.0, 1.0), ambient=0.05, diffuse=0.4, phong=0.8, phong_size=80.0,
                                   pattern=pattern))
    s.sphere((-4.0, 0.0, 0.0), 1.0, glass(Pattern("checker", [(0, (1.0, 1.0, 1.0), 0.9, 0.0), (1, (0.8, 0.15, 0.1))],
                                                  [("scale", (0.45, 0.45, 0.45)), off])),
             Interior(ior=1.5))
    s.sphere((-1.6, 0.0, -0.5), 1.0,
             glass(Pattern("marble", [(0.0, (0.95, 0.95, 0.9)), (0.6, (0.9, 0.7, 0.5), 0.7, 0.0),
                                      (1.0, (0.6, 0.9, 0.7), 0.9, 0.1)],
                           [("scale", (0.5, 0.5, 0.5)), off], turbulence=(0.6, 0.6, 0.6))),
             Interior(ior=1.33))
    s.sphere((0.8, 0.0, 0.0), 1.0, glass(Pattern("gradient", [(0.0, (0.2, 0.3, 0.9)), (1.0, (0.9, 0.9, 1.0), 0.0, 0.8)],
                                                  [("scale", (2.0, 2.0, 2.0)), ("translate", (0.0, -1.0, 0.0))],
                                                  gradient=(0.0, 1.0, 0.0))),
             Interior(ior=1.0))
    s.sphere((3.2, 0.0, -0.5), 1.0, glass(Pattern("bozo", [(0.0, (0.95, 0.95, 1.0), 0.85, 0.0),
                                                           (0.7, (0.8, 0.85, 0.9), 0.5, 0.0), (1.0, (0.5, 0.5, 0.55))],
                                                  [("scale", (0.4, 0.4, 0.4)), off])),
             Interior(ior=1.4))
    s.sphere((-2.8, 2.6, 1.5), 0.9, glass(Pattern("crackle", [(0.0, (0.3, 0.2, 0.1)), (0.08, (0.9, 0.8, 0.5), 0.0, 0.7),
                                                              (1.0, (1.0, 1.0, 0.9), 0.0, 0.9)],
                                                  [("scale", (0.35, 0.35, 0.35)), off])),
             Interior(ior=1.0))
    s.add(Scene.n_box((1.0, 1.8, 1.0), (2.6, 3.4, 2.6),
                      glass(Pattern("onion", [(0.0, (0.9, 0.95, 1.0), 0.9, 0.0), (0.5, (0.4, 0.6, 0.9), 0.6, 0.0),
                                              (1.0, (0.9, 0.95, 1.0), 0.9, 0.0)],
                                    [("scale", (0.5, 0.5, 0.5)), ("translate", (1.8, 2.6, 1.8))])),
                      interior=Interior(ior=1.3)))
    return s


def backlit_sheets(width=320, height=240):
    """Back-side diffuse light (finish { diffuse A, B }): thin boxes
    (translucent sheets, diffuse 0.5, 0.4) and spheres (diffuse 0.6, 0.3,
    phong 0.5) between the camera and a point light behind them, a second
    light in front, a box with plain diffuse for contrast, over a floor
    plane y=-1.5; camera (0,1.5,-9) looking at (0,0.5,0), 50 deg."""
    s = Scene("backlit_sheets", width, height, (0.0, 1.5, -9.0), (0.0, 0.5, 0.0), 50.0, max_trace_level=3)
    s.point_light((1.0, 4.0, 8.0), (1.2, 1.1, 0.9))
    s.point_light((-6.0, 5.0, -6.0), (0.4, 0.4, 0.45))
    s.plane((0.0, 1.0, 0.0), -1.5, s.material(Material((0.7, 0.75, 0.7))))
    leaf = s.material(Material((0.4, 0.8, 0.3), ambient=0.05, diffuse=0.5, diffuse_back=0.4))
    paper = s.material(Material((0.95, 0.9, 0.8), ambient=0.05, diffuse=0.5, diffuse_back=0.6))
    s.add(Scene.n_box((-3.5, -1.0, 1.0), (-1.5, 2.0, 1.05), leaf))
    s.add(Scene.n_box((1.2, -0.5, 0.5), (3.4, 2.5, 0.55), paper))
    s.add(Scene.n_box((-0.9, -1.0, 2.0), (0.9, 1.0, 2.05), s.material(Material((0.9, 0.3, 0.3)))))
    for c, r, rgb in (((-2.5, 0.0, -1.5), 0.7, (0.9, 0.6, 0.2)), ((0.2, 0.3, -2.0), 0.6, (0.3, 0.5, 0.9)),
                      ((2.3, 0.0, -1.0), 0.8, (0.8, 0.8, 0.8))):
        s.sphere(c, r, s.material(Material(rgb, diffuse=0.6, diffuse_back=0.3, phong=0.5)))
    return s


def metal_spheres(width=320, height=240):
    """Metallic finishes: spheres of gold, copper, steel and a painted
    metal with phong or specular highlights tinted by `metallic` (1, 0.8,
    0.5) and reflections tinted by reflection's `metallic` (0.9, 0.6), a
    plain reflective sphere for contrast, over a checker floor; two point
    lights; camera (0,3,-10) looking at (0,0.5,0), 50 deg;
    max_trace_level 4."""
    s = Scene("metal_spheres", width, height, (0.0, 3.0, -10.0), (0.0, 0.5, 0.0), 50.0, max_trace_level=4)
    s.point_light((6.0, 10.0, -8.0))
    s.point_light((-8.0, 6.0, -4.0), (0.5, 0.5, 0.55))
    floor = Pattern("checker", [(0.0, (0.85, 0.85, 0.8)), (1.0, (0.25, 0.3, 0.4))],
                    [("translate", (0.0, 0.5, 0.0))])
    s.plane((0.0, 1.0, 0.0), -1.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    for c, rgb, kw in (((-3.3, 0.0, 1.0), (0.95, 0.75, 0.3), dict(phong=0.9, phong_size=60.0, metallic=1.0,
                                                                   reflection=0.5, reflect_metallic=0.9)),
                       ((-1.1, 0.0, 0.0), (0.85, 0.45, 0.3), dict(specular=0.8, roughness=0.02, metallic=0.8,
                                                                   reflection=0.4, reflect_metallic=0.6)),
                       ((1.1, 0.0, 0.0), (0.7, 0.72, 0.75), dict(phong=0.7, metallic=0.5, reflection=0.35)),
                       ((3.3, 0.0, 1.0), (0.2, 0.5, 0.25), dict(phong=0.6, specular=0.4, metallic=1.0)),
                       ((0.0, 0.2, 2.8), (0.9, 0.9, 0.9), dict(phong=0.5, reflection=0.3))):
        s.sphere(c, 1.0, s.material(Material(rgb, diffuse=0.5, **kw)))
    return s


def bumpy_spheres(width=320, height=240, n_spheres=12, seed=7, noise_generator=None, waves=False):
    """Normal perturbation: a bumpy (scale 0.5, amount 0.3), mirror-ish
    (reflection 0.2) grey floor (plane y=-2) and `n_spheres` spheres r
    U[0.5,1.2] in a 6x6 area (seed 7) cycling through bumps (scale 0.2),
    dents (amount 0.8), wrinkles, granite (scale 2), marble and wood with
    turbulence, agate, onion, leopard, a sine-wave gradient, bozo with
    accuracy 0.05 and bumps with no_bump_scale under a rotation and a
    non-uniform scale; every sphere has phong 0.6, specular 0.3 and
    reflection 0.25 and a plain or bozo pigment; one point light; camera
    (0,3,-10) looking at (0,0,2), 55 deg; max_trace_level 3.  With `waves`
    the spheres alternate ripples and waves normals (frequency, phase,
    scale) over ripples and waves pigments."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("bumpy_spheres", width, height, (0.0, 3.0, -10.0), (0.0, 0.0, 2.0), 55.0, max_trace_level=3)
    s.point_light((10.0, 15.0, -10.0))
    ng = noise_generator
    floor_n = Normal(Pattern("bumps", [], [("scale", (0.5, 0.5, 0.5))], noise_generator=ng), amount=0.3)
    s.plane((0.0, 1.0, 0.0), -2.0, s.material(Material((0.6, 0.6, 0.65), reflection=0.2, normal=floor_n)))
    normals = [
        Normal(Pattern("bumps", [], [("scale", (0.2, 0.2, 0.2))], noise_generator=ng), amount=0.6),
        Normal(Pattern("dents", [], [("scale", (0.3, 0.3, 0.3))], noise_generator=ng), amount=0.8),
        Normal(Pattern("wrinkles", [], [("scale", (0.4, 0.4, 0.4))]), amount=0.5),
        Normal(Pattern("granite", [], [("scale", (2.0, 2.0, 2.0))], noise_generator=ng), amount=0.4),
        Normal(Pattern("marble", [], [("scale", (0.8, 0.8, 0.8))], turbulence=(0.7, 0.7, 0.7), noise_generator=ng),
               amount=0.7),
        Normal(Pattern("wood", [], [("scale", (0.15, 0.15, 0.15)), ("rotate", (90.0, 0.0, 0.0))],
                       turbulence=(0.05, 0.05, 0.05)), amount=0.5),
        Normal(Pattern("agate", [], [("scale", (0.5, 0.5, 0.5))], agate_turb=0.8, noise_generator=ng), amount=0.4),
        Normal(Pattern("onion", [], [("scale", (0.3, 0.3, 0.3))]), amount=0.6),
        Normal(Pattern("leopard", [], [("scale", (0.1, 0.1, 0.1))]), amount=0.5),
        Normal(Pattern("gradient", [], gradient=(1.0, 1.0, 0.0), wave="sine", frequency=2.0, phase=0.25), amount=0.8),
        Normal(Pattern("bozo", [], [("scale", (0.5, 0.5, 0.5))], noise_generator=ng), amount=0.6, accuracy=0.05),
        Normal(Pattern("bumps", [], [("scale", (0.3, 0.15, 0.3)), ("rotate", (30.0, 0.0, 20.0))], noise_generator=ng),
               amount=0.7, no_bump_scale=True),
    ]
    pig = Pattern("bozo", [(0.0, (0.9, 0.3, 0.1)), (0.5, (0.95, 0.9, 0.3)), (1.0, (0.1, 0.5, 0.2))],
                  [("scale", (0.4, 0.4, 0.4))], noise_generator=ng)
    if waves:
        normals = [
            Normal(Pattern("ripples", [], [("scale", (0.5, 0.5, 0.5))], frequency=3.0), amount=0.8),
            Normal(Pattern("waves", [], [("scale", (0.3, 0.3, 0.3)), ("translate", (0.2, 0.0, 0.1))],
                           frequency=2.0, phase=0.3), amount=0.6),
            Normal(Pattern("ripples", [], [("rotate", (0.0, 30.0, 0.0))], phase=0.5), amount=1.2),
            Normal(Pattern("waves", [], [("scale", (0.6, 0.6, 0.6))]), amount=0.9, no_bump_scale=True),
        ]
        pig = Pattern("ripples", [(0.0, (0.1, 0.2, 0.6)), (1.0, (0.9, 0.95, 1.0))], [("scale", (0.3, 0.3, 0.3))],
                      frequency=2.0)
        floor_pig = Pattern("waves", [(0.0, (0.2, 0.4, 0.3)), (0.5, (0.8, 0.8, 0.6)), (1.0, (0.3, 0.2, 0.1))],
                            [("scale", (0.7, 0.7, 0.7))], frequency=1.5, phase=0.2)
        s.materials[0].pattern = floor_pig
    for i in range(n_spheres):
        c = (rng.uniform(-3.0, 3.0), rng.uniform(-1.0, 1.5), rng.uniform(0.0, 6.0))
        r = rng.uniform(0.5, 1.2)
        rgb = tuple(float(x) for x in rng.uniform(0.3, 1.0, size=3))
        s.sphere(c, r, s.material(Material(rgb, phong=0.6, specular=0.3, reflection=0.25,
                                           pattern=pig if i % 3 == 0 else None,
                                           normal=normals[i % len(normals)])))
    return s


def shaped_spheres(width=320, height=240, n_spheres=12, seed=8, noise_generator=None):
    """Geometric and noise pigments: a boxed-pattern floor (plane y=-2,
    scale 3) and `n_spheres` spheres r U[0.5,1.2] in a 6x6 area (seed 8)
    cycling through radial (frequency 6), planar, spherical (scale 1.2,
    centred on the sphere), cylindrical, boxed, dents, wrinkles, square,
    triangular, cubic (centred on the sphere) and hexagon pigments,
    half of them with a radial or spherical slope normal; phong 0.4; one
    point light; camera (0,3,-10) looking at (0,0,2), 55 deg;
    max_trace_level 2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("shaped_spheres", width, height, (0.0, 3.0, -10.0), (0.0, 0.0, 2.0), 55.0, max_trace_level=2)
    s.point_light((10.0, 15.0, -10.0))
    ng = noise_generator
    warm = [(0.0, (0.9, 0.85, 0.7)), (0.6, (0.6, 0.3, 0.15)), (1.0, (0.2, 0.1, 0.05))]
    cool = [(0.0, (0.05, 0.1, 0.3)), (0.5, (0.5, 0.7, 0.9)), (1.0, (1.0, 1.0, 1.0))]
    floor = Pattern("boxed", cool, [("scale", (3.0, 3.0, 3.0))], wave="sine", frequency=2.0)
    s.plane((0.0, 1.0, 0.0), -2.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    for i in range(n_spheres):
        c = (rng.uniform(-3.0, 3.0), rng.uniform(-1.0, 1.5), rng.uniform(0.0, 6.0))
        r = rng.uniform(0.5, 1.2)
        at = [("translate", c)]
        kinds = [
            Pattern("radial", warm, [("rotate", (90.0, 0.0, 0.0))] + at, frequency=6.0),
            Pattern("planar", cool, [("scale", (r, r, r))] + at),
            Pattern("spherical", warm, [("scale", (1.2 * r, 1.2 * r, 1.2 * r))] + at),
            Pattern("cylindrical", cool, [("scale", (r, r, r))] + at, wave="scallop"),
            Pattern("boxed", warm, [("scale", (0.8 * r, 0.8 * r, 0.8 * r))] + at, wave="cubic"),
            Pattern("dents", cool, [("scale", (0.3, 0.3, 0.3))], noise_generator=ng),
            Pattern("wrinkles", warm, [("scale", (0.5, 0.5, 0.5))], noise_generator=ng),
            Pattern("square", [(k, rgb) for k, rgb in enumerate(((0.9, 0.2, 0.2), (0.2, 0.9, 0.2), (0.2, 0.2, 0.9),
                                                                  (0.9, 0.9, 0.2)))], [("scale", (0.3, 0.3, 0.3))]),
            Pattern("triangular", [(k, (0.15 * k + 0.1, 0.9 - 0.12 * k, 0.5)) for k in range(6)],
                    [("scale", (0.25, 0.25, 0.25)), ("rotate", (90.0, 0.0, 0.0))]),
            Pattern("cubic", [(k, (0.5, 0.15 * k + 0.1, 0.9 - 0.12 * k)) for k in range(6)], at),
            Pattern("hexagon", [(0, (0.9, 0.8, 0.2)), (1, (0.2, 0.6, 0.9)), (2, (0.8, 0.2, 0.5))],
                    [("scale", (0.2, 0.2, 0.2)), ("rotate", (-70.0, 0.0, 0.0))]),
        ]
        nrm = None
        if i % 2 == 1:
            nrm = Normal(Pattern("radial" if i % 4 == 1 else "spherical", [], at, frequency=8.0), amount=0.6)
        s.sphere(c, r, s.material(Material((1.0, 1.0, 1.0), phong=0.4, pattern=kinds[i % len(kinds)], normal=nrm)))
    return s


def patterned_spheres(width=320, height=240, n_spheres=12, seed=9, noise_generator=None):
    """The brick, spiral, cells, crackle and quilted patterns: a brick wall (plane z=9, brick
    size <0.8,0.3,0.5>, mortar 0.04), a cells floor (plane y=-2, scale
    0.7), and `n_spheres` spheres r U[0.5,1.1] in a 6x6 area (seed 9)
    cycling through spiral1 (3 arms), spiral2 (5 arms), cells (scale 0.3,
    sine wave), brick (size <0.3,0.12,0.2>, mortar 0.02), spiral1 with
    turbulence (0.3, octaves 4), cells with frequency 3, crackle, solid
    crackle, crackle with form <0.8,0.3,0>, metric 1 and offset 0.1, and
    quilted (control0 0.6, control1 0.9), the odd ones with a spiral2,
    cells or crackle slope normal; every pattern translated off
    the lattice so no surface lies on a cell or mortar boundary; phong
    0.4; one point light; camera (0,3,-10) looking at (0,0,2), 55 deg;
    max_trace_level 2."""
    rng = np.random.Generator(np.random.PCG64(seed))
    s = Scene("patterned_spheres", width, height, (0.0, 3.0, -10.0), (0.0, 0.0, 2.0), 55.0, max_trace_level=2)
    s.point_light((10.0, 15.0, -10.0))
    ng = noise_generator
    warm = [(0.0, (0.9, 0.85, 0.7)), (0.6, (0.6, 0.3, 0.15)), (1.0, (0.2, 0.1, 0.05))]
    cool = [(0.0, (0.05, 0.1, 0.3)), (0.5, (0.5, 0.7, 0.9)), (1.0, (1.0, 1.0, 1.0))]
    off = ("translate", (0.137, 0.071, 0.213))
    wall = Pattern("brick", [(0, (0.75, 0.75, 0.7)), (1, (0.6, 0.18, 0.1))], [off],
                   brick_size=(0.8, 0.3, 0.5), mortar=0.04)
    s.plane((0.0, 0.0, -1.0), -9.0, s.material(Material((1.0, 1.0, 1.0), pattern=wall)))
    floor = Pattern("cells", cool, [("scale", (0.7, 0.7, 0.7)), off])
    s.plane((0.0, 1.0, 0.0), -2.0, s.material(Material((1.0, 1.0, 1.0), pattern=floor)))
    for i in range(n_spheres):
        c = (rng.uniform(-3.0, 3.0), rng.uniform(-1.0, 1.5), rng.uniform(0.0, 6.0))
        r = rng.uniform(0.5, 1.1)
        at = [off, ("translate", c)]
        kinds = [
            Pattern("spiral1", warm, [("scale", (0.4, 0.4, 0.4))] + at, arms=3),
            Pattern("spiral2", cool, [("scale", (0.5, 0.5, 0.5)), ("rotate", (90.0, 0.0, 0.0))] + at, arms=5),
            Pattern("cells", warm, [("scale", (0.3, 0.3, 0.3)), off], wave="sine"),
            Pattern("brick", [(0, (0.9, 0.9, 0.85)), (1, (0.3, 0.5, 0.8))], [off], brick_size=(0.3, 0.12, 0.2),
                    mortar=0.02),
            Pattern("spiral1", cool, [("scale", (0.5, 0.5, 0.5))] + at, arms=2, turbulence=(0.3, 0.3, 0.3),
                    octaves=4, noise_generator=ng),
            Pattern("cells", cool, [("scale", (0.45, 0.45, 0.45)), off], frequency=3.0),
            Pattern("crackle", warm, [("scale", (0.35, 0.35, 0.35)), off]),
            Pattern("crackle", cool, [("scale", (0.4, 0.4, 0.4)), off], solid=True, noise_generator=ng),
            Pattern("crackle", warm, [("scale", (0.3, 0.3, 0.3)), off], form=(0.8, 0.3, 0.0), metric=1.0,
                    offset=0.1),
            Pattern("quilted", cool, [("scale", (0.3, 0.3, 0.3)), off], control0=0.6, control1=0.9),
        ]
        nrm = None
        if i % 2 == 1:
            nk = ("spiral2", "cells", "crackle")[(i // 2) % 3]
            nrm = Normal(Pattern(nk, [], [("scale", (0.3, 0.3, 0.3))] + at, arms=4), amount=0.5)
        s.sphere(c, r, s.material(Material((1.0, 1.0, 1.0), phong=0.4, pattern=kinds[i % len(kinds)], normal=nrm)))
    return s


VIEW_SIZES = ((256, 256), (640, 480), (1280, 720), (1920, 1080))


def circle_views(n_views=64, radius=30.0, y=5.0, seed=5, sizes=VIEW_SIZES):
    """`n_views` cameras evenly spaced on a circle of `radius` at height `y`,
    all looking at the origin; each view's resolution drawn uniformly from
    `sizes` (seed 5).  Returns [(location, look_at, width, height)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pick = rng.integers(0, len(sizes), size=n_views)
    views = []
    for i in range(n_views):
        a = 2.0 * math.pi * i / n_views
        loc = (radius * math.sin(a), y, -radius * math.cos(a))
        w, h = sizes[int(pick[i])]
        views.append((loc, (0.0, 0.0, 0.0), int(w), int(h)))
    return views


def view_of(scene, location, look_at, width, height):
    """The same scene seen from another camera at another resolution (what
    a View with its own camera renders), as a Scene of its own."""
    v = copy.copy(scene)
    v.location = tuple(float(x) for x in location)
    v.look_at = tuple(float(x) for x in look_at)
    v.width = int(width)
    v.height = int(height)
    v.right_len = float(width) / float(height)
    return v


def multiview_media(mesh_n=296, n_spheres=10000, seed=5, box=12.5, radiosity=True, count=200,
                    recursion_limit=2, error_bound=0.5, intervals=10, samples=10, scattering=0.05):
    """The batched multi-view scene: the displaced sphere mesh2 of
    mesh_spheres (radius 8, seed 2) + `n_spheres` spheres r U[0.1,0.5] in
    [-12,12]^3 (seed 5) + plane y=-9, one point light (20,30,-20), reflection
    0.3, max_trace_level 3; a uniform scattering media box [-box,box]^3
    (scattering rgb 0.05, intervals 10, samples 10, method 3) around it; with
    `radiosity`, radiosity { count 200 recursion_limit 2 error_bound 0.5 }.
    Its views come from circle_views (64 cameras, r 30, y 5)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-12.0, 12.0, size=(n_spheres, 3))
    radii = rng.uniform(0.1, 0.5, size=n_spheres)
    colours = rng.uniform(0.0, 1.0, size=(n_spheres, 3))
    s = Scene("multiview_media", 1920, 1080, (0.0, 5.0, -30.0), (0.0, 0.0, 0.0), 50.0, max_trace_level=3)
    s.point_light((20.0, 30.0, -20.0))
    s.media_box((-box, -box, -box), (box, box, box), scattering=(scattering,) * 3, intervals=intervals,
                samples=samples)
    mesh = displaced_sphere_mesh(n=mesh_n, seed=2)
    s.mesh(mesh, s.material(Material((0.9, 0.7, 0.4), phong=0.5, reflection=0.3)))
    for i in range(n_spheres):
        s.sphere(centres[i], radii[i], s.material(Material(colours[i], phong=0.5, reflection=0.3)))
    s.plane((0.0, 1.0, 0.0), -9.0, s.material(Material((0.8, 0.8, 0.8), phong=0.5, reflection=0.3)))
    if radiosity:
        s.radiosity = dict(count=count, recursion_limit=recursion_limit, error_bound=error_bound)
    return s


WORKLOADS = {
    "spheres_plane": spheres_plane,
    "mesh_spheres": mesh_spheres,
    "csg_torus_grid": csg_torus_grid,
    "radiosity_room": radiosity_room,
    "media_spheres": media_spheres,
    "multiview_media": multiview_media,
    "textured_spheres": textured_spheres,
    "bumpy_spheres": bumpy_spheres,
    "shaped_spheres": shaped_spheres,
    "glass_spheres": glass_spheres,
}
