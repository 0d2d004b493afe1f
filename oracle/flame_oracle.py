"""ORACLE -- test infrastructure only.

Python side of the CPU restatement of the reference's buffer path: builds
oracle/_build/liboracle.so from chaos_oracle.c, parses and normalises flame
JSON exactly as the reference does, and fills the flat ``or_flame``
description that the C code iterates.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg import this module; the product never does.

Reference behaviour restated here (file:line in the reference project):
  * JSON with // and /* */ comments (src/utils/json.cpp:15-23);
  * Flame(Json) validation, src/types/flame.hpp:91-210: size 1..65535
    (truncated from a number), bounds within +-1e10 with lo < hi,
    color_dimensions an integer <= 127, color_speed in [0,1], >= 1 xform;
  * XForm(Json), src/types/xform.hpp:71-172: weight >= 0, optional affines,
    colour length/range, per-xform color_speed, zero-weight variations
    dropped (xform.hpp:55-66);
  * Affine(Json) / Point(Json), src/types/affine.hpp:45-92,
    src/types/point.hpp:60-77;
  * Flame::_optimize (flame.hpp:63-83): zero-weight xforms dropped, the rest
    ordered by decreasing weight.  std::sort is an insertion sort (stable)
    for up to 16 elements in libstdc++; this restatement uses a stable sort
    for every size, so tie order can differ from the reference only for
    more than 16 xforms with equal weights;
  * Flame::_setupCumulativeWeights (flame.hpp:44-60);
  * Variation::parseVariation (src/variations/variations.hpp:2614-2626):
    2-D names first (only for dims >= 2), then N-D names.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import subprocess
import threading
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")

MAXD = 4
MAXC = 128
MAXX = 4096
NPARAM = 16

# variation name table: N-D names (variations.hpp:2567-2612) then 2-D names
# (variations.hpp:2387-2548); the id is the index in this list.
ND_NAMES = [
    "linear", "sinusoidal", "spherical", "bent", "rectangles", "fisheye",
    "bubble", "noise", "blur", "gaussian_blur", "square_noise", "separation",
    "splits", "pre_blur", "modulus", "celln", "spherical_p", "unit_sphere",
    "unit_sphere_p", "unit_cube",
]
TWO_D_NAMES = [
    "swirl", "horseshoe", "polar", "polar2", "handkerchief", "heart", "disc",
    "disc2", "waves", "fan", "rings", "spiral", "hyperbolic", "diamond", "ex",
    "julia", "exponential", "power", "cosine", "blob", "pdj", "cylinder",
    "perspective", "julian", "juliascope", "radial_blur", "pie", "ngon",
    "curl", "arch", "tangent", "rays", "blade", "secant", "twintrian",
    "cross", "exp", "log", "sin", "cos", "tan", "sec", "csc", "cot", "sinh",
    "cosh", "tanh", "sech", "csch", "coth", "auger", "flux", "mobius", "scry",
    "split", "stripes", "wedge", "wedge_julia", "wedge_sph", "whorl",
    "supershape", "flower", "conic", "parabola", "bipolar", "boarders",
    "butterfly", "cell", "cpow", "curve", "edisc", "elliptic", "escher",
    "foci", "lazysusan", "loonie", "oscope", "popcorn",
]
ALL_NAMES = ND_NAMES + TWO_D_NAMES
VAR_ID = {n: i for i, n in enumerate(ALL_NAMES)}

M_PI = 3.141592653589793
M_PI_2 = 1.5707963267948966
M_1_PI = 0.3183098861837907        # the double nearest 1/pi (glibc M_1_PI)
EPS = 1e-20


def _fdiv(a: float, b: float) -> float:
    """IEEE double division (inf/nan instead of ZeroDivisionError)."""
    with np.errstate(all="ignore"):
        return float(np.float64(a) / np.float64(b))


def _sin(x):
    with np.errstate(all="ignore"):
        return float(np.sin(np.float64(x))) if not math.isfinite(x) else math.sin(x)


def _cos(x):
    with np.errstate(all="ignore"):
        return float(np.cos(np.float64(x))) if not math.isfinite(x) else math.cos(x)


def rng_words(name: str, dims: int) -> int:
    """RNG words one call draws (FlameRNG draw counts, flame_rng.hpp)."""
    dw = 2 if dims == 3 else (2 * ((dims + 1) // 2) if dims > 3 else 1)
    if name in ("noise", "blur"):
        return 1 + dw
    if name in ("gaussian_blur", "pre_blur"):
        return 2 + dw
    if name == "square_noise":
        return dims
    if name in ("julia", "julian", "arch", "rays", "blade", "twintrian",
                "wedge_julia", "supershape", "flower", "conic", "boarders", "cpow"):
        return 1
    if name in ("juliascope", "radial_blur", "parabola"):
        return 2
    if name == "pie":
        return 3
    return 0


def _f(j, k, name):
    return float_value(key(j, k, name), f"{name}: {k}")


def _pt(j, k, n, name):
    return point_value(key(j, k, name), n, f"{name}: {k}")


def _params(name: str, j, dims: int) -> list:
    """Constructor arithmetic of each variation class (variations.hpp)."""
    f = lambda k: _f(j, k, name)
    if name in ("linear", "sinusoidal", "spherical", "noise", "blur",
                "gaussian_blur", "square_noise", "pre_blur", "unit_sphere",
                "unit_cube"):
        return []
    if name == "bent":                                   # 216-240
        return _pt(j, "scales_neg", dims, name) + _pt(j, "scales_pos", dims, name)
    if name in ("rectangles", "splits"):                 # 245-270, 410-429
        return _pt(j, "params", dims, name)
    if name in ("fisheye", "bubble"):                    # 275-314
        return [f("addval")]
    if name == "separation":                             # 383-405
        sep = _pt(j, "params", dims, name)
        return [v * v for v in sep] + _pt(j, "inside", dims, name)
    if name == "modulus":                                # 451-471
        p2 = [v * 2.0 for v in _pt(j, "params", dims, name)]
        return p2 + [_fdiv(1.0, v) for v in p2]
    if name == "celln":                                  # 476-505
        sz = _pt(j, "sizes", dims, name)
        return sz + [_fdiv(1.0, v) for v in sz]
    if name in ("spherical_p", "unit_sphere_p"):         # 2312-2363
        n = f("norm")
        if n <= 0.0:
            raise FlameError("norm <= 0")
        return [n]
    if name in ("swirl", "horseshoe", "polar", "polar2", "handkerchief", "heart",
                "disc", "spiral", "hyperbolic", "diamond", "ex", "julia",
                "exponential", "power", "cosine", "cylinder", "tangent", "cross",
                "exp", "log", "sin", "cos", "tan", "sec", "csc", "cot", "sinh",
                "cosh", "tanh", "sech", "csch", "coth", "butterfly", "edisc",
                "elliptic", "foci"):
        return []
    if name == "disc2":                                  # 624-655
        rot, twist = f("rotation"), f("twist")
        rotpi = rot * M_PI
        sinadd, cosadd = _sin(twist), _cos(twist)
        cosadd -= 1.0
        k = 1.0 + twist
        if twist > 2.0 * M_PI:
            k -= 2.0 * M_PI
        if twist < -2.0 * M_PI:
            k += 2.0 * M_PI
        return [rotpi, cosadd * k, sinadd * k]
    if name == "waves":                                  # 660-680
        return [f("xfreq"), f("xscale"), f("yfreq"), f("yscale")]
    if name == "fan":                                    # 685-709
        x, y = f("x"), f("y")
        return [M_PI * (x * x + EPS), y]
    if name == "rings":                                  # 714-733
        v = f("value")
        return [v * v + EPS]
    if name == "blob":                                   # 875-896
        low, high = f("low"), f("high")
        return [(high + low) / 2.0, (high - low) / 2.0, f("waves")]
    if name == "pdj":                                    # 901-925
        return [f("a"), f("b"), f("c"), f("d")]
    if name == "perspective":                            # 943-962
        dist, ang = f("distance"), f("angle")
        return [dist, _sin(ang), dist * _cos(ang)]
    if name in ("julian", "juliascope"):                 # 967-1018
        power, dist = f("power"), f("dist")
        return [abs(power), _fdiv(1.0, power), _fdiv(dist, 2.0 * power)]
    if name == "radial_blur":                            # 1023-1045
        ang = f("angle")
        a = ang * M_PI_2
        return [_sin(a), _cos(a), f("flam3_weight")]
    if name == "pie":                                    # 1050-1072
        slices, rot, thick = f("slices"), f("rotation"), f("thickness")
        return [slices, rot, thick, _fdiv(2.0 * M_PI, slices)]
    if name == "ngon":                                   # 1077-1102
        sides = f("sides")
        powerval = f("power") / 2.0
        ang = _fdiv(2.0 * M_PI, sides)
        corners, circle = f("corners"), f("circle")
        return [powerval, ang, corners, circle, sides / (2.0 * M_PI)]
    if name == "curl":                                   # 1107-1129
        return [f("c1"), f("c2")]
    if name in ("arch", "rays", "blade", "secant", "twintrian", "scry"):
        return [f("flam3_weight")]
    if name == "auger":                                  # 1549-1571
        freq, w = f("freq"), f("flam3_weight")
        return [freq, w, f("scale") / 2.0, f("sym")]
    if name == "flux":                                   # 1576-1600
        return [2.0 + f("spread"), f("flam3_weight")]
    if name == "mobius":                                 # 1605-1630
        out = []
        for k in ("a", "b", "c", "d"):
            out += _pt(j, k, 2, name)
        return out
    if name == "split":                                  # 1655-1673
        return [f("xsize") * M_PI, f("ysize") * M_PI]
    if name == "stripes":                                # 1678-1696
        return [1.0 - f("space"), f("warp")]
    if name == "wedge":                                  # 1701-1724
        swirl, count, ang, hole = f("swirl"), f("count"), f("angle"), f("hole")
        return [swirl, count, ang, hole, 1.0 - ang * count * (M_1_PI * 0.5)]
    if name == "wedge_julia":                            # 1729-1756
        ang, count, power = f("angle"), f("count"), f("power")
        invpower = _fdiv(1.0, power)
        dist = f("dist")
        cn = _fdiv(dist, 2.0 * power)
        return [ang, count, invpower, cn, abs(power),
                1.0 - ang * count * (M_1_PI * 0.5)]
    if name == "wedge_sph":                              # 1761-1785
        ang, count, swirl, hole = f("angle"), f("count"), f("swirl"), f("hole")
        return [ang, count, swirl, hole, 1.0 - ang * count * (M_1_PI * 0.5)]
    if name == "whorl":                                  # 1790-1810
        return [f("inside"), f("outside"), f("flam3_weight")]
    if name == "supershape":                             # 1815-1842
        n1 = f("n1")
        pm_4 = f("m") / 4.0
        return [pm_4, _fdiv(-1.0, n1), f("n2"), f("n3"), f("rnd"), f("holes")]
    if name == "flower":                                 # 1847-1864
        return [f("petals"), f("holes")]
    if name == "conic":                                  # 1869-1886
        return [f("eccen"), f("holes")]
    if name == "parabola":                               # 1891-1909
        return [f("height"), f("width")]
    if name == "bipolar":                                # 1914-1935
        return [-M_PI_2 * f("shift")]
    if name == "boarders":                               # 1940-1983
        prob = f("prob")
        if prob < 0.0 or prob > 1.0:
            raise FlameError("boarders probability out of range")
        return [prob]
    if name == "cell":                                   # 2008-2033
        size = f("size")
        return [size, _fdiv(1.0, size)]
    if name == "cpow":                                   # 2038-2061
        r, i, power = f("r"), f("i"), f("power")
        return [_fdiv(2.0 * M_PI, power), _fdiv(r, power), _fdiv(i, power), power]
    if name == "curve":                                  # 2066-2091
        xamp, yamp, xlen, ylen = f("xamp"), f("yamp"), f("xlen"), f("ylen")
        xlen *= xlen
        ylen *= ylen
        mx = xlen if EPS < xlen else EPS
        my = ylen if EPS < ylen else EPS
        return [xamp, yamp, 1.0 / mx, 1.0 / my]
    if name == "escher":                                 # 2149-2171
        beta = f("beta")
        return [0.5 * (1.0 + _cos(beta)), 0.5 * _sin(beta)]
    if name == "lazysusan":                              # 2197-2230
        return [f("x"), f("y"), f("spin"), f("twist"), f("space"), f("flam3_weight")]
    if name == "loonie":                                 # 2235-2254
        w = f("flam3_weight")
        return [w, w * w]
    if name == "oscope":                                 # 2259-2281
        freq = f("frequency")
        return [2.0 * M_PI * freq, f("amplitude"), f("damping"), f("separation")]
    if name == "popcorn":                                # 2286-2305
        return [f("x"), f("y"), f("c")]
    raise FlameError(f"unknown variation: {name}")


class FlameError(ValueError):
    """Flame JSON rejected (the reference throws JsonError / runtime_error)."""


# --------------------------------------------------------------- JSON
def strip_comments(text: str) -> str:
    out = []
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if c == '"':
            j = i + 1
            while j < n and text[j] != '"':
                j += 2 if text[j] == "\\" else 1
            out.append(text[i:j + 1])
            i = j + 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            if j < 0:
                raise FlameError("json: unterminated comment")
            out.append(" ")
            i = j + 2
        else:
            out.append(c)
            i += 1
    return "".join(out)


def _reject_constant(name):
    raise FlameError(f"json: invalid literal {name}")


def parse_json(text: str):
    try:
        return json.loads(strip_comments(text), parse_constant=_reject_constant)
    except json.JSONDecodeError as e:
        raise FlameError(f"json: {e}") from None


def _is_int(v) -> bool:
    return type(v) is int


def _is_num(v) -> bool:
    return type(v) is int or type(v) is float


def float_value(v, what: str) -> float:
    if not _is_num(v):
        raise FlameError(f"{what}: type is not float")
    return float(v)


def int_value(v, what: str) -> int:
    if not _is_int(v):
        raise FlameError(f"{what}: type is not int")
    return v


def key(obj, k: str, what: str):
    if not isinstance(obj, dict):
        raise FlameError(f"{what}: not an object")
    if k not in obj:
        raise FlameError(f"{what}: key does not exist: {k}")
    return obj[k]


def point_value(v, n: int, what: str) -> list[float]:
    if not isinstance(v, list):
        raise FlameError(f"{what}: not an array")
    if len(v) != n:
        raise FlameError(f"{what}: incorrect array size: {len(v)}")
    out = []
    for e in v:
        if not _is_num(e):
            raise FlameError(f"{what}: entry is not a number")
        out.append(float(e))
    return out


# --------------------------------------------------------------- model
@dataclass
class Var:
    name: str
    weight: float
    axis_x: int = 0
    axis_y: int = 1
    params: list = field(default_factory=list)

    @property
    def type(self) -> int:
        return VAR_ID[self.name]


@dataclass
class XForm:
    id: int
    weight: float
    has_pre: bool
    pre_A: list
    pre_b: list
    has_post: bool
    post_A: list
    post_b: list
    vars: list
    color: list
    color_speed: float


@dataclass
class Flame:
    dims: int
    size: list
    bounds: list
    color_dims: int
    color_speed: float
    xforms: list            # sorted, zero weights removed
    removed: list
    xform_ids: int
    final: XForm | None
    xfcw: list


def _affine(j, n: int, what: str):
    if not isinstance(j, dict):
        raise FlameError(f"{what}: not an object")
    if "A" in j:
        A = j["A"]
        if not isinstance(A, list):
            raise FlameError(f"{what}: A is not an array")
        if len(A) != n:
            raise FlameError(f"{what}: A is wrong size")
        rows = [point_value(r, n, f"{what}: A[{i}]") for i, r in enumerate(A)]
    else:
        rows = [[1.0 if i == k else 0.0 for k in range(n)] for i in range(n)]
    b = point_value(j["b"], n, f"{what}: b") if "b" in j else [0.0] * n
    return [x for r in rows for x in r], b


def _identity(n: int):
    return [1.0 if i == k else 0.0 for i in range(n) for k in range(n)], [0.0] * n


def parse_variation(j, dims: int) -> Var:
    name = key(j, "name", "variation")
    if not isinstance(name, str):
        raise FlameError("variation: name is not a string")
    is2d = name in TWO_D_NAMES and dims >= 2
    if not is2d and name not in ND_NAMES:
        raise FlameError(f"unknown variation: {name}")
    weight = float_value(key(j, "weight", "variation"), "variation weight")
    v = Var(name=name, weight=weight)
    v.params = _params(name, j, dims)
    if is2d and dims > 2:
        ax = int_value(key(j, "axis_x", name), "axis_x")
        ay = int_value(key(j, "axis_y", name), "axis_y")
        if ax < 0 or ax >= dims:
            raise FlameError("axis_x index out of range")
        if ay < 0 or ay >= dims:
            raise FlameError("axis_y index out of range")
        if ax == ay:
            raise FlameError("axes are not distinct")
        v.axis_x, v.axis_y = ax, ay
    return v


def parse_xform(j, xid: int, is_final: bool, dims: int, color_dims: int,
                default_speed: float) -> XForm:
    if not is_final:
        weight = float_value(key(j, "weight", "XForm()"), "XForm(): weight")
    else:
        weight = 1.0
    if weight < 0.0:
        raise FlameError("XForm(): weight is negative")
    if not isinstance(j, dict):
        raise FlameError("XForm(): not an object")
    has_pre = "pre_affine" in j
    pre = _affine(j["pre_affine"], dims, "pre_affine") if has_pre else _identity(dims)
    has_post = "post_affine" in j
    post = _affine(j["post_affine"], dims, "post_affine") if has_post else _identity(dims)
    varsj = key(j, "variations", "XForm()")
    if not isinstance(varsj, list):
        raise FlameError("XForm(): variations is not an array")
    vs = [parse_variation(v, dims) for v in varsj]
    color = []
    if color_dims and "color" in j:
        cj = j["color"]
        if not isinstance(cj, list):
            raise FlameError("XForm(): color is not an array")
        if len(cj) != color_dims:
            raise FlameError("XForm(): color length incorrect")
        for c in cj:
            c = float_value(c, "color")
            if c < 0.0 or c > 1.0:
                raise FlameError("XForm(): color coordinate out of range")
            color.append(c)
    if color_dims and "color_speed" in j:
        speed = float_value(j["color_speed"], "color_speed")
        if speed < 0.0 or speed > 1.0:
            raise FlameError("XForm(): color speed out of range")
    else:
        speed = default_speed
    vs = [v for v in vs if abs(v.weight) != 0.0]
    return XForm(id=xid, weight=weight, has_pre=has_pre, pre_A=pre[0],
                 pre_b=pre[1], has_post=has_post, post_A=post[0],
                 post_b=post[1], vars=vs, color=color, color_speed=speed)


def load_flame(text_or_obj) -> Flame:
    j = parse_json(text_or_obj) if isinstance(text_or_obj, str) else text_or_obj
    dims = int_value(key(j, "dimensions", "flame"), "dimensions")
    if dims < 1 or dims > MAXD:
        raise FlameError(f"{dims}D not supported")
    sizej = key(j, "size", "Flame()")
    boundsj = key(j, "bounds", "Flame()")
    if not isinstance(sizej, list) or not isinstance(boundsj, list):
        raise FlameError("Flame(): size/bounds not arrays")
    if len(sizej) != dims:
        raise FlameError("Flame(): incorrect size length")
    if len(boundsj) != dims:
        raise FlameError("Flame(): incorrect bounds length")
    size, bounds = [], []
    for i in range(dims):
        s = float_value(sizej[i], f"size[{i}]")
        if not (s >= 1.0) or s >= 65536.0:
            raise FlameError(f"Flame(): size[{i}] out of range")
        s = int(math.trunc(s))
        b = boundsj[i]
        if not isinstance(b, list) or len(b) != 2:
            raise FlameError(f"Flame(): bounds[{i}] wrong format")
        lo = float_value(b[0], f"bounds[{i}]")
        hi = float_value(b[1], f"bounds[{i}]")
        M = 1e10
        if lo < -M or lo > M or hi < -M or hi > M:
            raise FlameError(f"Flame(): bounds[{i}] out of range")
        if lo >= hi:
            raise FlameError(f"Flame(): bounds[{i}] low >= high")
        size.append(s)
        bounds.append((lo, hi))
    xfs = key(j, "xforms", "Flame()")
    if not isinstance(xfs, list):
        raise FlameError("Flame(): cannot parse xforms")
    color_dims = int_value(j["color_dimensions"], "color_dimensions") \
        if "color_dimensions" in j else 0
    if color_dims < 0 or color_dims > 127:
        raise FlameError("Flame(): too many color dimensions")
    speed = float_value(j["color_speed"], "color_speed") if "color_speed" in j else 0.5
    if speed < 0.0 or speed > 1.0:
        raise FlameError("Flame(): color speed out of range")
    xforms = [parse_xform(x, i, False, dims, color_dims, speed)
              for i, x in enumerate(xfs)]
    if not xforms:
        raise FlameError("Flame(): no xforms")
    final = None
    if "final_xform" in j:
        final = parse_xform(j["final_xform"], (1 << 64) - 1, True, dims,
                            color_dims, speed)
    kept = [x for x in xforms if x.weight != 0.0]
    removed = [x for x in xforms if x.weight == 0.0]
    if not kept:
        raise FlameError("Flame(): no xforms remaining after optimization")
    kept.sort(key=lambda x: -x.weight)
    normdiv = 0.0
    for x in kept:
        normdiv += x.weight
    xfcw, wsum = [], 0.0
    for x in kept:
        wsum += x.weight / normdiv
        xfcw.append(wsum)
    xfcw[-1] = 1.0
    return Flame(dims=dims, size=size, bounds=bounds, color_dims=color_dims,
                 color_speed=speed, xforms=kept, removed=removed,
                 xform_ids=len(xforms), final=final, xfcw=xfcw)


def index_mults(fl: Flame):
    """BufferRenderer::_init (buffer_renderer.hpp:114-140)."""
    mult_d, mult_i, cells = [], [], 1
    for i in range(fl.dims):
        lo, hi = fl.bounds[i]
        m = float(fl.size[i]) / (hi - lo)
        m *= 1.0 - 2.0 ** -52
        mult_d.append(m)
        mult_i.append(cells)
        cells *= fl.size[i]
    return mult_d, mult_i, cells


# --------------------------------------------------------------- ctypes
class OrVar(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("axis_x", ctypes.c_int32),
                ("axis_y", ctypes.c_int32), ("rng_draws", ctypes.c_int32),
                ("weight", ctypes.c_double),
                ("params", ctypes.c_double * NPARAM)]


class OrXForm(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("weight", ctypes.c_double),
                ("has_pre", ctypes.c_int32), ("has_post", ctypes.c_int32),
                ("pre_A", ctypes.c_double * (MAXD * MAXD)),
                ("pre_b", ctypes.c_double * MAXD),
                ("post_A", ctypes.c_double * (MAXD * MAXD)),
                ("post_b", ctypes.c_double * MAXD),
                ("var_begin", ctypes.c_int32), ("var_count", ctypes.c_int32),
                ("has_color", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("color_speed", ctypes.c_double)]


class OrFlame(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int32), ("nxf", ctypes.c_int32),
                ("has_final", ctypes.c_int32), ("color_dims", ctypes.c_int32),
                ("xform_ids", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("size", ctypes.c_uint64 * MAXD),
                ("lo", ctypes.c_double * MAXD), ("hi", ctypes.c_double * MAXD),
                ("xf", ctypes.POINTER(OrXForm)), ("vars", ctypes.POINTER(OrVar)),
                ("colors", ctypes.POINTER(ctypes.c_double)),
                ("xfcw", ctypes.POINTER(ctypes.c_double))]


class OrStats(ctypes.Structure):
    _fields_ = [("ok", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("s_iter", ctypes.c_uint64), ("s_plot", ctypes.c_uint64),
                ("bad", ctypes.c_uint64), ("dropped", ctypes.c_uint64),
                ("ext_lo", ctypes.c_double * MAXD),
                ("ext_hi", ctypes.c_double * MAXD),
                ("xf_dist", ctypes.c_uint64 * MAXX)]


class OracleFlame:
    """A Flame packed into the C layout; keeps the backing arrays alive."""

    def __init__(self, fl: Flame):
        self.flame = fl
        n = fl.dims
        allx = list(fl.xforms) + ([fl.final] if fl.final else [])
        nv = sum(len(x.vars) for x in allx)
        self._vars = (OrVar * max(nv, 1))()
        self._xf = (OrXForm * (len(fl.xforms) + 1))()
        self._colors = (ctypes.c_double * max((len(fl.xforms) + 1) * fl.color_dims, 1))()
        self._xfcw = (ctypes.c_double * len(fl.xfcw))(*fl.xfcw)
        vi = 0
        for k, x in enumerate(allx):
            cx = self._xf[k]
            cx.id = x.id
            cx.weight = x.weight
            cx.has_pre, cx.has_post = int(x.has_pre), int(x.has_post)
            for i in range(n * n):
                cx.pre_A[i] = x.pre_A[i]
                cx.post_A[i] = x.post_A[i]
            for i in range(n):
                cx.pre_b[i] = x.pre_b[i]
                cx.post_b[i] = x.post_b[i]
            cx.var_begin, cx.var_count = vi, len(x.vars)
            cx.has_color = int(bool(x.color))
            cx.color_speed = x.color_speed
            for c, val in enumerate(x.color):
                self._colors[k * fl.color_dims + c] = val
            for v in x.vars:
                cv = self._vars[vi]
                cv.type, cv.axis_x, cv.axis_y = v.type, v.axis_x, v.axis_y
                cv.rng_draws = rng_words(v.name, n)
                cv.weight = v.weight
                for p, val in enumerate(v.params):
                    cv.params[p] = val
                vi += 1
        self.c = OrFlame()
        self.c.dims, self.c.nxf = n, len(fl.xforms)
        self.c.has_final = int(fl.final is not None)
        self.c.color_dims = fl.color_dims
        self.c.xform_ids = fl.xform_ids
        for i in range(n):
            self.c.size[i] = fl.size[i]
            self.c.lo[i], self.c.hi[i] = fl.bounds[i]
        self.c.xf = self._xf
        self.c.vars = self._vars
        self.c.colors = self._colors
        self.c.xfcw = self._xfcw


_lib = None
_lib_lock = threading.Lock()


def build(force: bool = False) -> str:
    """Compile chaos_oracle.c into oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "chaos_oracle.c")
    hdr = os.path.join(HERE, "chaos_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src),
                                                  os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off",
                           "-fno-fast-math", "-fPIC", "-shared", "-Wall",
                           "-o", tmp, src, "-lm", "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lib_lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            u64, i32, dp = ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p
            L.oracle_isaac_words.argtypes = [u64, u64, dp]
            L.oracle_fmix64.argtypes = [u64]
            L.oracle_fmix64.restype = u64
            L.oracle_stream_key.argtypes = [u64, u64]
            L.oracle_stream_key.restype = u64
            L.oracle_pick_sequence.argtypes = [ctypes.POINTER(OrFlame), u64, u64, dp]
            L.oracle_step.argtypes = [ctypes.POINTER(OrFlame), i32, u64, u64, dp, dp]
            L.oracle_render.argtypes = [ctypes.POINTER(OrFlame), u64, u64, u64,
                                        u64, u64, u64, ctypes.c_int, dp, dp,
                                        ctypes.POINTER(OrStats)]
            L.oracle_trace.argtypes = [ctypes.POINTER(OrFlame), u64, u64, u64, dp, dp]
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def isaac_words(key_: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint64)
    lib().oracle_isaac_words(key_, n, _ptr(out))
    return out


def stream_key(seed: int, stream: int) -> int:
    return lib().oracle_stream_key(seed, stream)


def pick_sequence(of: OracleFlame, key_: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.int32)
    lib().oracle_pick_sequence(ctypes.byref(of.c), key_, n, _ptr(out))
    return out


def step(of: OracleFlame, xf_index: int, key_: int, pts: np.ndarray) -> np.ndarray:
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros_like(pts)
    rc = lib().oracle_step(ctypes.byref(of.c), xf_index, key_,
                           pts.shape[0], _ptr(pts), _ptr(out))
    if rc != 0:
        raise ValueError("oracle_step: bad xform index")
    return out


def trace(of: OracleFlame, key_: int, settle: int, n: int):
    ids = np.zeros(n, dtype=np.int32)
    pts = np.zeros((n, of.flame.dims), dtype=np.float64)
    lib().oracle_trace(ctypes.byref(of.c), key_, settle, n, _ptr(ids), _ptr(pts))
    return ids, pts


@dataclass
class RenderResult:
    counts: np.ndarray          # uint64 [cells]
    colors: np.ndarray          # float64 [cells, color_dims]
    ok: bool
    s_iter: int
    s_plot: int
    bad: int
    dropped: int
    xf_dist: np.ndarray
    ext_lo: np.ndarray
    ext_hi: np.ndarray

    def file_bytes(self) -> bytes:
        """Reference buffer file layout (buffer_renderer.hpp:476-480)."""
        cells = self.counts.shape[0]
        r = self.colors.shape[1]
        out = np.zeros((cells, 1 + r), dtype=np.uint64)
        out[:, 0] = self.counts
        if r:
            out[:, 1:] = self.colors.view(np.uint64)
        return out.tobytes()


def render(of: OracleFlame, seed: int, streams: int, samples: int,
           traj_len: int, settle: int, bad_limit: int = 256,
           threads: int = 1) -> RenderResult:
    fl = of.flame
    _, _, cells = index_mults(fl)
    counts = np.zeros(cells, dtype=np.uint64)
    colors = np.zeros((cells, fl.color_dims), dtype=np.float64)
    st = OrStats()
    rc = lib().oracle_render(ctypes.byref(of.c), seed, streams, samples,
                             traj_len, settle, bad_limit, threads,
                             _ptr(counts), _ptr(colors), ctypes.byref(st))
    if rc != 0:
        raise ValueError("oracle_render: bad arguments")
    n = fl.dims
    return RenderResult(counts=counts, colors=colors, ok=bool(st.ok),
                        s_iter=st.s_iter, s_plot=st.s_plot, bad=st.bad,
                        dropped=st.dropped,
                        xf_dist=np.array(st.xf_dist[:fl.xform_ids], dtype=np.uint64),
                        ext_lo=np.array(st.ext_lo[:n]), ext_hi=np.array(st.ext_hi[:n]))


def oracle_flame_from_file(path: str) -> OracleFlame:
    with open(path, "r", encoding="utf-8") as f:
        return OracleFlame(load_flame(f.read()))
