"""Scene description: a Python mirror of the reference's ShapeTree API and the serializer
front end that turns a Scene into the piles the raster kernels read.

Reference semantics (file:line):
  STree / SRep / Scene / Compound        Figure/ShapeTree.hs:84-176
  overlap = foldl combine emptyItem      Layout/Adjacent.hs:183-190  (first item is front-most)
  cAdd = SMeld CompoundAdd               Layout/Draw.hs:62-64
  cSubtract = flip (SMeld CompoundSubtract)  (the subtracted shape sits above)
  traverseTree (above first; transforms compose inner-first)   Raster/TraverseShapeTree.hs:44-80
  compound inversion under Subtract      Raster/TraverseShapeTree.hs:35-37
  segmentsToCurvePairs (straight -> midpoint control)          Figure/Outline.hs:95-103
  Transformer application                Figure/Transformer.hs:87-98
  picture usage transform                Figure/Picture.hs:116-122

All coordinates are float32 and every transform is applied in float32 one step at a
time, as the reference does with Float.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Any, List, Optional, Sequence

import numpy as np

from . import lib as L

# ------------------------------------------------------------------ geometry


class Outline:
    """A closed loop of curve pairs (onCurve, offCurve) -- Figure/Outline.hs Outline."""

    __slots__ = ("pairs",)

    def __init__(self, pairs):
        p = np.asarray(pairs, dtype=np.float32).reshape(-1, 4)
        self.pairs = np.ascontiguousarray(p)

    def __len__(self):
        return self.pairs.shape[0]


def straight(x, y):
    return (np.float32(x), np.float32(y), None)


def curved(x, y, cx, cy):
    return (np.float32(x), np.float32(y), (np.float32(cx), np.float32(cy)))


def segments_to_outline(segments: Sequence) -> Outline:
    """segmentsToCurvePairs (Figure/Outline.hs:95-103): a straight segment gets the
    midpoint of its anchor and the next anchor (cyclically) as its control point."""
    n = len(segments)
    pairs = np.zeros((n, 4), dtype=np.float32)
    half = np.float32(0.5)
    for i, (x, y, c) in enumerate(segments):
        pairs[i, 0] = x
        pairs[i, 1] = y
        if c is None:
            nx, ny, _ = segments[(i + 1) % n]
            # lerp 0.5 v0 v1 = 0.5*v0 + (1-0.5)*v1 in Float
            pairs[i, 2] = half * np.float32(x) + half * np.float32(nx)
            pairs[i, 3] = half * np.float32(y) + half * np.float32(ny)
        else:
            pairs[i, 2] = c[0]
            pairs[i, 3] = c[1]
    return Outline(pairs)


# ------------------------------------------------------------------ trees

ADD = 0
SUBTRACT = 1


@dataclass
class Translate:
    dx: float
    dy: float


@dataclass
class Scale:
    s: float


@dataclass
class Rotate:
    """Rotation by an angle in radians (not used by the benchmark scenes; cos/sin are
    evaluated in float32 by numpy)."""
    radians: float


@dataclass
class Leaf:
    rep: Any


@dataclass
class Meld:
    op: Any          # ADD / SUBTRACT for compound trees, None (overlap) for shape trees
    above: Any
    below: Any


@dataclass
class Transform:
    xform: Any
    child: Any


class _Empty:
    def __repr__(self):
        return "SEmpty"


EMPTY = _Empty()


@dataclass
class Solid:
    color: Sequence[float]  # sRGB-encoded RGBA floats


@dataclass
class Texture:
    picture: str


@dataclass
class Radial:
    center: Sequence[float]
    radius: float
    inner: Sequence[float]
    outer: Sequence[float]


@dataclass
class SRep:
    token: int
    substance: Any
    compound: Any  # compound tree whose leaves are lists of Outlines


@dataclass
class Picture:
    """RGBA8 bitmap (height, width, 4) uint8 -- Figure/Picture.hs PictureImage."""
    pixels: np.ndarray


@dataclass
class Scene:
    background: Sequence[float]
    tree: Any
    pictures: dict = field(default_factory=dict)


def shape(outlines: Sequence[Outline]):
    """A compound leaf made of outlines (fromSegments / SLeaf)."""
    return Leaf(list(outlines))


def cAdd(a, b):
    return Meld(ADD, a, b)


def cSubtract(a, b):
    """Subtract b from a: b is placed above a with the subtract combinator."""
    return Meld(SUBTRACT, b, a)


def solid(color, compound, token=0):
    return Leaf(SRep(token, Solid(tuple(float(c) for c in color)), compound))


def texture_with(picture_name, compound, token=0):
    return Leaf(SRep(token, Texture(picture_name), compound))


def radial_with(center, radius, inner, outer, compound, token=0):
    return Leaf(SRep(token, Radial(tuple(center), float(radius), tuple(inner), tuple(outer)), compound))


def overlap(items: Sequence):
    """foldl combine emptyItem: the first item ends up front-most."""
    acc = EMPTY
    for it in items:
        acc = Meld(None, acc, it)
    return acc


def t_translate(dx, dy, tree):
    if np.float32(dx) == 0 and np.float32(dy) == 0:
        return tree
    return Transform(Translate(np.float32(dx), np.float32(dy)), tree)


def t_scale(s, tree):
    if np.float32(s) == 1:
        return tree
    return Transform(Scale(np.float32(s)), tree)


def t_rotate(radians, tree):
    if radians == 0:
        return tree
    return Transform(Rotate(radians), tree)


# ------------------------------------------------------------------ flattening


def _apply_points(xforms: List, pts: np.ndarray) -> np.ndarray:
    """Apply transforms innermost first (CombineTransform a b = b . a)."""
    out = pts.astype(np.float32, copy=True)
    for xf in xforms:  # innermost first
        if isinstance(xf, Translate):
            out[:, 0] = out[:, 0] + np.float32(xf.dx)
            out[:, 1] = out[:, 1] + np.float32(xf.dy)
        elif isinstance(xf, Scale):
            out = out * np.float32(xf.s)
        elif isinstance(xf, Rotate):
            c = np.float32(np.cos(np.float32(xf.radians)))
            s = np.float32(np.sin(np.float32(xf.radians)))
            x = out[:, 0].copy()
            y = out[:, 1].copy()
            out[:, 0] = x * c - y * s
            out[:, 1] = x * s + y * c
    return out


def _apply_usage(xforms: List, translate, scale):
    """PictureUsage transform (Figure/Picture.hs:116-122): translate adds, scale
    multiplies the scale, rotation is ignored."""
    tx, ty, sc = np.float32(translate[0]), np.float32(translate[1]), np.float32(scale)
    for xf in xforms:
        if isinstance(xf, Translate):
            tx = np.float32(np.float32(xf.dx) + tx)
            ty = np.float32(np.float32(xf.dy) + ty)
        elif isinstance(xf, Scale):
            sc = np.float32(np.float32(xf.s) * sc)
    return tx, ty, sc


@dataclass
class FlatScene:
    canvas_w: int
    canvas_h: int
    background: np.ndarray
    substance_kind: np.ndarray
    substance_color: np.ndarray
    substance_picture: np.ndarray
    substance_picture_xform: np.ndarray
    substance_radial: np.ndarray
    substance_shape_start: np.ndarray
    shape_compound: np.ndarray
    shape_outline_start: np.ndarray
    outline_pair_start: np.ndarray
    pairs: np.ndarray
    pictures: np.ndarray          # picture pile bytes
    picture_size: np.ndarray
    picture_offset: np.ndarray
    # the scene's name of each picture in the pile (None: the pictures are numbered)
    picture_names: Optional[list] = None


class PictureLibrary:
    """Pictures packed once into one RGBA8 pile that stays on the device across
    frames.

    The reference packs the scene's whole picture map into a fresh pile, and uploads
    it, for every frame (makePictData, Figure/Picture.hs:159-167, from queueRasterJobs,
    OpenCL/CallKernels.hs:228-240).  Here every picture gets a fixed 4-byte aligned
    offset in one pile, uploaded once (Rasterizer.upload_pictures); bind() points a
    scene's picture usages at those offsets, so a frame uploads only its own piles
    (Rasterizer.upload_frame).  Texels are read exactly as from a per-frame pile."""

    def __init__(self, pictures):
        """pictures: a mapping from names to Picture (or (h, w, 4) uint8 arrays), or a
        sequence of them named 0, 1, ..."""
        items = pictures.items() if hasattr(pictures, "items") else enumerate(pictures)
        self.offsets: dict = {}
        self.sizes: dict = {}
        chunks, off = [], 0
        for key, p in items:
            px = np.ascontiguousarray(getattr(p, "pixels", p), dtype=np.uint8)
            if px.ndim != 3 or px.shape[2] != 4:
                raise ValueError(f"picture {key!r} is not an (h, w, 4) RGBA8 bitmap")
            self.offsets[key] = off
            self.sizes[key] = (int(px.shape[1]), int(px.shape[0]))
            chunks.append(px.reshape(-1))
            off += px.size
        if off > np.iinfo(np.int32).max:
            raise ValueError("picture pile beyond 2 GB (offsets are 32-bit)")
        self.pile = np.concatenate(chunks) if chunks else np.zeros(0, np.uint8)

    def bind(self, flat: "FlatScene") -> "FlatScene":
        """The same scene with its pictures looked up in this library: usages point
        into the library's pile and the scene carries no picture bytes of its own."""
        import dataclasses
        n = int(flat.picture_offset.size)
        names = list(flat.picture_names) if flat.picture_names is not None else list(range(n))
        sizes, offsets = [], []
        for i, key in enumerate(names):
            if key not in self.offsets:
                raise KeyError(f"cannot find picture {key!r} in the picture library")
            if tuple(int(v) for v in flat.picture_size[i]) != self.sizes[key]:
                raise ValueError(f"picture {key!r} differs in size from the library's")
            sizes.append(self.sizes[key])
            offsets.append(self.offsets[key])
        return dataclasses.replace(
            flat, pictures=np.zeros(0, np.uint8),
            picture_size=np.asarray(sizes, dtype=np.int32).reshape(-1, 2),
            picture_offset=np.asarray(offsets, dtype=np.int32), picture_names=names)


def flatten(scene: Scene, canvas_w: int, canvas_h: int) -> FlatScene:
    """Walk the shape tree the way traverseShapeTree / traverseCompoundTree do and
    collect substances, compound leaves and outlines in traversal order."""
    kinds, colors, pics, pxf, radials, sub_start = [], [], [], [], [], [0]
    compounds, outline_start, pair_start, pair_chunks = [], [0], [0], []
    pic_names: dict = {}
    pic_list: list = []
    n_pairs = 0

    def visit_compound(node, comp, xforms):
        nonlocal n_pairs
        if node is EMPTY:
            return
        if isinstance(node, Leaf):
            outlines = node.rep
            compounds.append(comp)
            for o in outlines:
                pts = o.pairs.reshape(-1, 2)
                if xforms:
                    pts = _apply_points(xforms, pts)
                pair_chunks.append(np.ascontiguousarray(pts.reshape(-1, 4), dtype=np.float32))
                n_pairs += pts.shape[0] // 2
                pair_start.append(n_pairs)
            outline_start.append(len(pair_start) - 1)
        elif isinstance(node, Meld):
            if node.op == SUBTRACT:
                visit_compound(node.above, SUBTRACT if comp == ADD else ADD, xforms)
            else:
                visit_compound(node.above, comp, xforms)
            visit_compound(node.below, comp, xforms)
        elif isinstance(node, Transform):
            visit_compound(node.child, comp, [node.xform] + xforms)
        else:
            raise TypeError(f"unexpected compound node {node!r}")

    def on_srep(rep: "SRep", xforms):
        sub = rep.substance
        if isinstance(sub, Solid):
            kinds.append(0)
            colors.append(np.asarray(sub.color, dtype=np.float32))
            pics.append(0)
            pxf.append((0.0, 0.0, 1.0))
            radials.append(None)
        elif isinstance(sub, Texture):
            if sub.picture not in scene.pictures:
                raise KeyError(f"cannot find picture name {sub.picture!r} in picture map")
            if sub.picture not in pic_names:
                pic_names[sub.picture] = len(pic_list)
                pic_list.append(scene.pictures[sub.picture])
            kinds.append(1)
            colors.append(np.zeros(4, np.float32))
            pics.append(pic_names[sub.picture])
            pxf.append(_apply_usage(xforms, (0.0, 0.0), 1.0))
            radials.append(None)
        elif isinstance(sub, Radial):
            c = np.asarray([sub.center], np.float32)
            if xforms:
                c = _apply_points(xforms, c)
            r = np.float32(sub.radius)
            for xf in xforms:
                if isinstance(xf, Scale):
                    r = np.float32(r * np.float32(xf.s))
            kinds.append(2)
            colors.append(np.zeros(4, np.float32))
            pics.append(0)
            pxf.append((0.0, 0.0, 1.0))
            radials.append((float(c[0, 0]), float(c[0, 1]), float(r), tuple(sub.inner), tuple(sub.outer)))
        else:
            raise TypeError(f"unknown substance {sub!r}")
        visit_compound(rep.compound, ADD, xforms)
        sub_start.append(len(compounds))

    # the overlap tree can be thousands of levels deep: walk it with an explicit stack,
    # above before below
    stack = [(scene.tree, [])]
    while stack:
        node, xforms = stack.pop()
        if node is EMPTY:
            continue
        if isinstance(node, Leaf):
            on_srep(node.rep, xforms)
        elif isinstance(node, Meld):
            stack.append((node.below, xforms))
            stack.append((node.above, xforms))
        elif isinstance(node, Transform):
            stack.append((node.child, [node.xform] + xforms))
        else:
            raise TypeError(f"unexpected shape node {node!r}")


    n_sub = len(kinds)
    rad = np.zeros(n_sub, dtype=L.RADIAL_DTYPE)
    for i, r in enumerate(radials):
        if r is not None:
            rad[i]["center_x"], rad[i]["center_y"], rad[i]["radius"] = r[0], r[1], r[2]
            rad[i]["inner"] = r[3]
            rad[i]["outer"] = r[4]
    # picture pile: pictures in order of first use (makePictData, Figure/Picture.hs:159-167)
    sizes, offsets, chunks, off = [], [], [], 0
    for p in pic_list:
        px = np.ascontiguousarray(p.pixels, dtype=np.uint8)
        h, w = px.shape[0], px.shape[1]
        sizes.append((w, h))
        offsets.append(off)
        chunks.append(px.reshape(-1))
        off += px.size
    pairs = np.concatenate(pair_chunks) if pair_chunks else np.zeros((0, 4), np.float32)
    return FlatScene(
        canvas_w=int(canvas_w), canvas_h=int(canvas_h),
        background=np.asarray(scene.background, dtype=np.float32),
        substance_kind=np.asarray(kinds, dtype=np.int32),
        substance_color=np.ascontiguousarray(np.asarray(colors, dtype=np.float32).reshape(-1, 4)),
        substance_picture=np.asarray(pics, dtype=np.int32),
        substance_picture_xform=np.ascontiguousarray(np.asarray(pxf, dtype=np.float32).reshape(-1, 3)),
        substance_radial=rad,
        substance_shape_start=np.asarray(sub_start, dtype=np.int32),
        shape_compound=np.asarray(compounds, dtype=np.int32),
        shape_outline_start=np.asarray(outline_start, dtype=np.int32),
        outline_pair_start=np.asarray(pair_start, dtype=np.int32),
        pairs=np.ascontiguousarray(pairs, dtype=np.float32),
        pictures=np.concatenate(chunks) if chunks else np.zeros(0, np.uint8),
        picture_size=np.asarray(sizes, dtype=np.int32).reshape(-1, 2),
        picture_offset=np.asarray(offsets, dtype=np.int32),
        picture_names=list(pic_names),
    )


def bake_radials(flat: FlatScene) -> FlatScene:
    """The same scene with every radial-gradient substance replaced by an RGBA8
    picture of the gradient over its shapes' bounding box: the reference's only route
    for a gradient (a PictureFunction evaluated on the host into a bitmap,
    Figure/Picture.hs:59-73), whose kernels know solid colours and pictures only
    (Kernels.cl readColor, K:1411-1442).  Texels are the gradient at integer pixel
    positions, as the radial substance evaluates it, rounded to 8 bits, so the two
    renderings agree within one LSB per channel."""
    kinds = flat.substance_kind.copy()
    pics = flat.substance_picture.copy()
    pxf = flat.substance_picture_xform.copy()
    sizes = [tuple(s) for s in flat.picture_size.reshape(-1, 2)]
    offsets = list(flat.picture_offset.astype(np.int64))
    chunks = [flat.pictures]
    off = int(flat.pictures.size)
    pts = flat.pairs.reshape(-1, 2)
    for i in np.nonzero(kinds == 2)[0]:
        s0, s1 = flat.substance_shape_start[i], flat.substance_shape_start[i + 1]
        o0, o1 = flat.shape_outline_start[s0], flat.shape_outline_start[s1]
        p0, p1 = flat.outline_pair_start[o0], flat.outline_pair_start[o1]
        p = pts[2 * p0:2 * p1]
        if p.size == 0:
            x0 = y0 = 0
            x1 = y1 = 1
        else:
            x0 = int(np.clip(np.floor(p[:, 0].min()), 0, flat.canvas_w - 1))
            y0 = int(np.clip(np.floor(p[:, 1].min()), 0, flat.canvas_h - 1))
            x1 = int(np.clip(np.ceil(p[:, 0].max()) + 1, x0 + 1, flat.canvas_w))
            y1 = int(np.clip(np.ceil(p[:, 1].max()) + 1, y0 + 1, flat.canvas_h))
        g = flat.substance_radial[i]
        ys, xs = np.mgrid[y0:y1, x0:x1].astype(np.float32)
        dx = xs - np.float32(g["center_x"])
        dy = ys - np.float32(g["center_y"])
        t = np.minimum(np.sqrt(dx * dx + dy * dy) / np.float32(g["radius"]), np.float32(1.0))
        inner, outer = g["inner"].astype(np.float32), g["outer"].astype(np.float32)
        rgba = inner[None, None, :] + (outer - inner)[None, None, :] * t[..., None]
        texels = np.clip(np.round(rgba * np.float32(255.0)), 0, 255).astype(np.uint8)
        kinds[i] = 1
        pics[i] = len(sizes)
        pxf[i] = (np.float32(x0), np.float32(y0), np.float32(1.0))
        sizes.append((x1 - x0, y1 - y0))
        offsets.append(off)
        chunks.append(texels.reshape(-1))
        off += texels.size
    return FlatScene(
        canvas_w=flat.canvas_w, canvas_h=flat.canvas_h, background=flat.background,
        substance_kind=kinds, substance_color=flat.substance_color, substance_picture=pics,
        substance_picture_xform=np.ascontiguousarray(pxf, dtype=np.float32),
        substance_radial=np.zeros(len(kinds), dtype=L.RADIAL_DTYPE),
        substance_shape_start=flat.substance_shape_start, shape_compound=flat.shape_compound,
        shape_outline_start=flat.shape_outline_start, outline_pair_start=flat.outline_pair_start,
        pairs=flat.pairs, pictures=np.concatenate(chunks),
        picture_size=np.asarray(sizes, dtype=np.int32).reshape(-1, 2),
        picture_offset=np.asarray(offsets, dtype=np.int32))


# ------------------------------------------------------------------ serialized frame


@dataclass
class Job:
    shapes: np.ndarray   # SHAPE_DTYPE
    tiles: np.ndarray    # TILE_DTYPE
    columns: int


@dataclass
class Frame:
    """Everything one frame hands to the raster kernels (the reference's
    BuffersInCommon plus its RasterJobs)."""
    canvas_w: int
    canvas_h: int
    spec: L.Spec
    background: np.ndarray
    geometry: np.ndarray       # uint8
    substances: np.ndarray     # float32 (n, 4)
    pictures: np.ndarray       # uint8
    picture_uses: np.ndarray   # PICTURE_USE_DTYPE
    radials: np.ndarray        # RADIAL_DTYPE
    random_field: np.ndarray   # float32 (4096,)
    jobs: List[Job]
    stats: dict
    # provenance of the geometry pile's points (see gudni_frame_point_*)
    point_offsets: Optional[np.ndarray] = None   # uint32 (n,)
    point_sources: Optional[np.ndarray] = None   # int32 (n, 3)
    point_weights: Optional[np.ndarray] = None   # float32 (n, 3)
    n_pairs: int = 0

    @property
    def compute_depth(self) -> int:
        return L.compute_depth(self.spec.threads_per_tile)

    @property
    def n_tiles(self) -> int:
        return sum(len(j.tiles) for j in self.jobs)


def default_random_field(seed: int = 0) -> np.ndarray:
    """4096 uniform floats in [0,1) (Util/RandomField.hs:27-30; seeded here)."""
    return np.random.default_rng(seed).random(L.RANDOM_FIELD_SIZE, dtype=np.float32)


def serialize(scene: Scene, canvas_w: int, canvas_h: int, spec: L.Spec,
              random_field: Optional[np.ndarray] = None) -> Frame:
    flat = flatten(scene, canvas_w, canvas_h)
    return serialize_flat(flat, spec, random_field)


def write_scene_file(path: str, flat: FlatScene, spec: L.Spec, random_field: Optional[np.ndarray] = None) -> None:
    """Write a flattened scene with its spec, picture pile and random field as the
    scene file gudni_render reads: a list of named arrays (u32 name length, name, u64
    byte count, bytes), the arrays of gudni_scene_desc under their field names."""
    arrays = {
        "header": np.array([flat.canvas_w, flat.canvas_h, flat.substance_kind.size, flat.picture_offset.size],
                           np.int32),
        "spec": np.frombuffer(bytes(spec), np.uint8),
        "background": np.asarray(flat.background, np.float32),
        "substance_kind": flat.substance_kind.astype(np.int32),
        "substance_color": flat.substance_color.astype(np.float32),
        "substance_picture": flat.substance_picture.astype(np.int32),
        "substance_picture_xform": flat.substance_picture_xform.astype(np.float32),
        "substance_radial": flat.substance_radial,
        "substance_shape_start": flat.substance_shape_start.astype(np.int32),
        "shape_compound": flat.shape_compound.astype(np.int32),
        "shape_outline_start": flat.shape_outline_start.astype(np.int32),
        "outline_pair_start": flat.outline_pair_start.astype(np.int32),
        "pairs": flat.pairs.astype(np.float32),
        "picture_size": flat.picture_size.astype(np.int32),
        "picture_offset": flat.picture_offset.astype(np.int32),
        "pictures": flat.pictures.astype(np.uint8),
        "random_field": np.asarray(default_random_field() if random_field is None else random_field, np.float32),
    }
    with open(path, "wb") as f:
        for name, a in arrays.items():
            b = np.ascontiguousarray(a).tobytes()
            f.write(np.uint32(len(name)).tobytes() + name.encode() + np.uint64(len(b)).tobytes() + b)


def scene_desc(flat: FlatScene):
    """The gudni_scene_desc of a flattened scene, and the arrays it points into (keep
    them alive while the descriptor is in use)."""
    d = L.SceneDesc()
    d.canvas_w, d.canvas_h = flat.canvas_w, flat.canvas_h
    for i in range(4):
        d.background[i] = float(flat.background[i])
    d.n_substances = int(flat.substance_kind.size)
    keep = []

    def a(arr):
        arr = np.ascontiguousarray(arr)
        keep.append(arr)
        return arr.ctypes.data if arr.size else None

    d.substance_kind = a(flat.substance_kind)
    d.substance_color = a(flat.substance_color)
    d.substance_picture = a(flat.substance_picture)
    d.substance_picture_xform = a(flat.substance_picture_xform)
    d.substance_radial = a(flat.substance_radial)
    d.substance_shape_start = a(flat.substance_shape_start)
    d.shape_compound = a(flat.shape_compound)
    d.shape_outline_start = a(flat.shape_outline_start)
    d.outline_pair_start = a(flat.outline_pair_start)
    d.pairs = a(flat.pairs)
    d.n_pictures = int(flat.picture_offset.size)
    d.picture_size = a(flat.picture_size)
    d.picture_offset = a(flat.picture_offset)
    return d, keep


def serialize_flat(flat: FlatScene, spec: L.Spec, random_field: Optional[np.ndarray] = None,
                   threads: int = 0) -> Frame:
    """Serialize a flattened scene.  threads == 1: the sequential restatement of the
    reference's walk (gudni_serialize); otherwise the same piles from the serializer's
    data-parallel passes on that many host threads, 0 for all (gudni_serialize_parallel)."""
    lib = L.load_host()
    d, keep = scene_desc(flat)
    if threads == 1:
        h = lib.gudni_serialize(C.byref(d), C.byref(spec))
    else:
        h = lib.gudni_serialize_parallel(C.byref(d), C.byref(spec), int(threads))
    if not h:
        raise ValueError("serialize failed: " + lib.gudni_serialize_error().decode())
    try:
        geo = L._copy(lib.gudni_frame_geometry(h), lib.gudni_frame_geometry_bytes(h), np.uint8)
        subs = L._copy(lib.gudni_frame_substances(h), lib.gudni_frame_n_substances(h), np.dtype((np.float32, 4)))
        uses = L._copy(lib.gudni_frame_picture_uses(h), lib.gudni_frame_n_picture_uses(h), L.PICTURE_USE_DTYPE)
        rads = L._copy(lib.gudni_frame_radials(h), lib.gudni_frame_n_radials(h), L.RADIAL_DTYPE)
        jobs = []
        for j in range(lib.gudni_frame_n_jobs(h)):
            shapes = L._copy(lib.gudni_frame_job_shapes(h, j), lib.gudni_frame_job_n_shapes(h, j), L.SHAPE_DTYPE)
            tiles = L._copy(lib.gudni_frame_job_tiles(h, j), lib.gudni_frame_job_n_tiles(h, j), L.TILE_DTYPE)
            jobs.append(Job(shapes, tiles, int(lib.gudni_frame_job_columns(h, j))))
        npts = lib.gudni_frame_n_points(h)
        p_off = L._copy(lib.gudni_frame_point_offsets(h), npts, np.uint32)
        p_src = L._copy(lib.gudni_frame_point_sources(h), 3 * npts, np.int32).reshape(-1, 3)
        p_w = L._copy(lib.gudni_frame_point_weights(h), 3 * npts, np.float32).reshape(-1, 3)
        st = (C.c_int64 * 8)()
        lib.gudni_frame_stats(h, st)
        stats = dict(zip(["shapes", "excluded", "strands", "tiles", "splits", "max_tile_shapes",
                          "max_tile_strands", "tile_shape_refs"], list(st)))
    finally:
        lib.gudni_frame_free(h)
    if random_field is None:
        random_field = default_random_field()
    return Frame(flat.canvas_w, flat.canvas_h, spec, flat.background.copy(), geo,
                 subs.reshape(-1, 4), flat.pictures.copy(), uses, rads,
                 np.ascontiguousarray(random_field, dtype=np.float32), jobs, stats,
                 p_off, p_src, p_w, int(flat.pairs.shape[0]))


def concatenated_piles(frame: Frame):
    """The frame's shape piles concatenated, tiles with their shape slices offset into
    the concatenation, and the job index of every tile (the layout of
    gudni_raster_tiles_device)."""
    shapes, tiles, jobs = [], [], []
    base = 0
    for j, job in enumerate(frame.jobs):
        shapes.append(job.shapes)
        t = job.tiles.copy()
        t["shape_start"] += np.uint32(base)
        tiles.append(t)
        jobs.append(np.full(len(t), j, np.int32))
        base += len(job.shapes)
    return (np.concatenate(shapes) if shapes else np.zeros(0, L.SHAPE_DTYPE),
            np.concatenate(tiles) if tiles else np.zeros(0, L.TILE_DTYPE),
            np.concatenate(jobs) if jobs else np.zeros(0, np.int32))


def pair_gradient(frame: Frame, grad_geometry: np.ndarray) -> np.ndarray:
    """Carry a gradient over the geometry pile's floats back to the scene's curve
    pairs ((n_pairs, 4): onCurve x, y, offCurve x, y) through the serializer's point
    provenance (knob splits are fixed linear combinations)."""
    g = np.zeros((frame.n_pairs * 2, 2), np.float64)
    off = frame.point_offsets.astype(np.int64)
    gx = np.asarray(grad_geometry, np.float64)[off]
    gy = np.asarray(grad_geometry, np.float64)[off + 1]
    for j in range(3):
        src = frame.point_sources[:, j]
        w = frame.point_weights[:, j].astype(np.float64)
        m = src >= 0
        np.add.at(g[:, 0], src[m], w[m] * gx[m])
        np.add.at(g[:, 1], src[m], w[m] * gy[m])
    return g.reshape(frame.n_pairs, 4)
