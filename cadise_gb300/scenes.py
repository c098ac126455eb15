"""Seeded procedural scenes in the reference's scene vocabulary.

A :class:`SceneSpec` holds exactly what a CRSD file holds (film, camera,
renderer, accelerator, light cluster, materials, primitives, lights) and can be
written out as CRSD text (``to_crsd``), the scene format parsed by the
reference (``source/file-io/scene-description/sdParser.cpp:19-35``,
``tokenizer.cpp:12-43``).  Large meshes are kept as numpy arrays so the same
scene can also be handed to the C-ABI as flat arrays without a text round trip.

Workloads
---------
* :func:`cornell_box` - the 5-wall Cornell box: 556-unit box with one quad per
  wall, a 165^3 box rotated -18 deg and a 165x330x165 box rotated 15 deg
  (12 triangles each), a 130x105 ceiling quad light with emission (17, 12, 4),
  white/red/green Lambert albedos, 40 deg pinhole, 256^2, 16 spp, depth 6.
* :func:`icosphere_field` - displaced icospheres over a 2-triangle ground plane
  with Lambert / GGX conductor / dielectric materials and quad area lights.
  With ``n_spheres=200, subdivision=4`` it is the 1,024,000-triangle field
  rendered at 1920x1080, 64 spp, depth 12.

Area-light mapping: an emission RGB ``E`` on a quad of area ``A`` is written as
``color "E"`` and ``watt = sum(E) * A * pi``, because the reference sets
``L = color / sum(color) * watt / (A * pi)``
(``source/core/light/category/singleAreaLight.cpp:32-36``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

# Material kinds understood by the CUDA library (and by the reference where a
# CRSD type exists for them).
LAMBERT = "matte-lambertian"
CONDUCTOR = "conductor-microfacet"
GLASS = "glass"
# Rough (GGX) dielectric after Walter et al. 2007.  The reference has no rough
# dielectric, so this type exists only in this library.
ROUGH_DIELECTRIC = "dielectric-microfacet"
MIRROR = "mirror"
PHONG = "phong"
PLASTIC = "plastic"


@dataclass
class Material:
    name: str
    type: str
    albedo: tuple = (0.5, 0.5, 0.5)
    roughness: float = 0.0
    f0: tuple = (1.0, 1.0, 1.0)
    ior_outer: float = 1.0
    ior_inner: float = 1.5
    albedo_texture: Optional[str] = None  # name of a texture-spectrum block
    exponent: float = 32.0            # phong "exponent", plastic "specular-exponent"
    diffuse_ratio: float = 0.7        # plastic "diffuse-ratio"
    fresnel: str = "conductor"        # mirror "fresnel-type": conductor (f0) or dielectric (iors)


@dataclass
class Rectangle:
    name: str
    material: str
    v1: tuple
    v2: tuple
    v3: tuple


@dataclass
class Triangle:
    """A single ``triangle`` primitive (can carry an area light)."""
    name: str
    material: str
    v1: tuple
    v2: tuple
    v3: tuple


@dataclass
class Sphere:
    name: str
    material: str
    center: tuple
    radius: float


@dataclass
class TriangleMesh:
    name: str
    material: str
    positions: np.ndarray  # (n_tri, 3, 3) float32
    normals: Optional[np.ndarray] = None  # (n_tri, 3, 3)
    uvws: Optional[np.ndarray] = None  # (n_tri, 3, 3)


@dataclass
class AreaLight:
    primitive: str
    color: tuple
    watt: float
    back_face_emit: bool = False


@dataclass
class ImageTexture:
    """RGB float texture, nearest lookup with repeat wrap.  Row 0 of
    `texels` is v = 0, the picture's bottom row (the reference lays every
    picture out that way: its loader flips images vertically)."""
    name: str
    texels: np.ndarray  # (h, w, 3) float32

    def write_pfm(self, path: str) -> None:
        """Portable float map: rows in file order from the bottom row up,
        which is the order of `texels`."""
        h, w, _ = self.texels.shape
        with open(path, "wb") as f:
            f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
            f.write(np.ascontiguousarray(self.texels, dtype="<f4").tobytes())


@dataclass
class FilmFilter:
    """Film reconstruction filter, CRSD film block keys (filterInstantiator.cpp:16-57):
    type box | gaussian | mitchell | cone; width / height default 1 for the box,
    4 for the others; tile = the film tile size clipping each sample's footprint."""
    type: str = "box"
    width: Optional[float] = None
    height: Optional[float] = None
    sigma_x: float = 0.5
    sigma_y: float = 0.5
    amplitude: float = 1.0
    b: float = 1.0 / 3.0
    c: float = 1.0 / 3.0
    tile: tuple = (16, 16)

    def size(self):
        d = 1.0 if self.type == "box" else 4.0
        return (self.width if self.width is not None else d, self.height if self.height is not None else d)


@dataclass
class SceneSpec:
    width: int
    height: int
    spp: int
    max_depth: int
    cam_position: tuple
    cam_direction: tuple
    cam_up: tuple
    fov: float
    sensor_width_mm: float = 36.0
    materials: List[Material] = field(default_factory=list)
    # primitives in CRSD order: Rectangle or TriangleMesh objects
    primitives: List[object] = field(default_factory=list)
    lights: List[AreaLight] = field(default_factory=list)
    textures: List[ImageTexture] = field(default_factory=list)
    # name of an ImageTexture used as a latitude-longitude environment light
    environment: Optional[str] = None
    # light selection: "uniform" (the reference's default) or "power"
    light_cluster: str = "uniform"
    # film filter; None: the box of size 1
    film_filter: Optional[FilmFilter] = None

    # ------------------------------------------------------------------ sizes
    def num_primitives(self) -> int:
        """Primitive count in the reference's sense (one per rectangle, one per
        mesh triangle), i.e. the length of its intersector list."""
        n = 0
        for p in self.primitives:
            n += 1 if isinstance(p, (Rectangle, Triangle, Sphere)) else int(p.positions.shape[0])
        return n

    def num_triangles(self) -> int:
        """Triangles after splitting every rectangle in two."""
        n = 0
        for p in self.primitives:
            if isinstance(p, Rectangle):
                n += 2
            elif isinstance(p, Triangle):
                n += 1
            else:
                n += int(p.positions.shape[0])
        return n

    # ------------------------------------------------------------------- CRSD
    def write_crsd(self, path: str, sidecar_min_triangles: int = 4096, header: str = "") -> None:
        """Write the scene as a CRSD file; meshes with at least
        `sidecar_min_triangles` triangles go to binary float32 sidecar files
        next to it (`[positions-file string ...]`) instead of text arrays, and
        image textures to PFM files next to it."""
        import os
        base = os.path.dirname(os.path.abspath(path))
        stem = os.path.splitext(os.path.basename(path))[0]
        with open(path, "w") as f:
            f.write(header)
            f.write(self.to_crsd(sidecar=(base, stem, sidecar_min_triangles)))

    def to_crsd(self, with_header: bool = True, sidecar=None) -> str:
        out: List[str] = []
        w = out.append

        def v3(v):
            return "%.9g %.9g %.9g" % (float(v[0]), float(v[1]), float(v[2]))

        f = self.film_filter or FilmFilter()
        fw, fh = f.size()
        w("film {\n    [image-width int32 \"%d\"]\n    [image-height int32 \"%d\"]\n"
          "    [filter string \"%s\"]\n" % (self.width, self.height, f.type))
        if (fw, fh) != ((1.0, 1.0) if f.type == "box" else (4.0, 4.0)):
            w("    [filter-width real \"%.9g\"]\n    [filter-height real \"%.9g\"]\n" % (fw, fh))
        if f.type == "gaussian":
            w("    [sigma-x real \"%.9g\"]\n    [sigma-y real \"%.9g\"]\n    [amplitude real \"%.9g\"]\n"
              % (f.sigma_x, f.sigma_y, f.amplitude))
        if f.type == "mitchell":
            w("    [b real \"%.9g\"]\n    [c real \"%.9g\"]\n" % (f.b, f.c))
        if tuple(f.tile) != (16, 16):
            w("    [tile-size-x int32 \"%d\"]\n    [tile-size-y int32 \"%d\"]\n" % tuple(f.tile))
        w("}\n")
        w("camera {\n    [type string \"perspective-pinhole\"]\n"
          "    [position vector3r \"%s\"]\n    [direction vector3r \"%s\"]\n"
          "    [up vector3r \"%s\"]\n    [fov real \"%.9g\"]\n"
          "    [sensor-width-mm real \"%.9g\"]\n}\n"
          % (v3(self.cam_position), v3(self.cam_direction), v3(self.cam_up),
             self.fov, self.sensor_width_mm))
        w("renderer {\n    [type string \"sampling\"]\n    [sample-number int32 \"%d\"]\n"
          "    [sampler string \"stratified\"]\n    [estimator string \"pt\"]\n"
          "    [max-depth int32 \"%d\"]\n}\n" % (self.spp, self.max_depth))
        w("accelerator {\n    [type string \"bvh\"]\n}\n")
        w("light-cluster {\n    [type string \"%s\"]\n}\n" % self.light_cluster)
        for t in self.textures:
            if t.name == self.environment:
                continue
            if sidecar is None:
                raise ValueError("image texture '%s' needs a PFM file next to the CRSD: use write_crsd" % t.name)
            import os
            base, stem, _ = sidecar
            fn = "%s.%s.pfm" % (stem, t.name)
            t.write_pfm(os.path.join(base, fn))
            w("texture-spectrum {\n    [type string \"image\"]\n    [name string \"%s\"]\n"
              "    [filename string \"%s\"]\n    [sample-mode string \"nearest\"]\n"
              "    [wrap-mode string \"repeat\"]\n}\n" % (t.name, fn))
        for m in self.materials:
            w("material {\n    [type string \"%s\"]\n    [name string \"%s\"]\n" % (m.type, m.name))
            if m.type == LAMBERT:
                if m.albedo_texture:
                    w("    [albedo texture \"%s\"]\n" % m.albedo_texture)
                else:
                    w("    [albedo rgb \"%s\"]\n" % v3(m.albedo))
            elif m.type == CONDUCTOR:
                w("    [microfacet-type string \"ggx\"]\n    [fresnel-type string \"schlick\"]\n"
                  "    [f0 rgb \"%s\"]\n    [roughness real \"%.9g\"]\n" % (v3(m.f0), m.roughness))
            elif m.type in (GLASS, ROUGH_DIELECTRIC):
                w("    [albedo rgb \"%s\"]\n    [ior-outer real \"%.9g\"]\n    [ior-inner real \"%.9g\"]\n"
                  % (v3(m.albedo), m.ior_outer, m.ior_inner))
                if m.type == ROUGH_DIELECTRIC:
                    w("    [roughness real \"%.9g\"]\n" % m.roughness)
            elif m.type == MIRROR:
                w("    [albedo rgb \"%s\"]\n    [fresnel-type string \"%s\"]\n" % (v3(m.albedo), m.fresnel))
                if m.fresnel == "conductor":
                    w("    [f0 rgb \"%s\"]\n" % v3(m.f0))
                else:
                    w("    [ior-outer real \"%.9g\"]\n    [ior-inner real \"%.9g\"]\n" % (m.ior_outer, m.ior_inner))
            elif m.type == PHONG:
                w("    [exponent real \"%.9g\"]\n" % m.exponent)
            elif m.type == PLASTIC:
                w("    [diffuse-albedo rgb \"%s\"]\n    [specular-exponent real \"%.9g\"]\n"
                  "    [diffuse-ratio real \"%.9g\"]\n" % (v3(m.albedo), m.exponent, m.diffuse_ratio))
            w("}\n")
        for p in self.primitives:
            if isinstance(p, Triangle):
                w("primitive {\n    [type string \"triangle\"]\n    [name string \"%s\"]\n"
                  "    [bsdf material \"%s\"]\n    [v1 vector3r \"%s\"]\n    [v2 vector3r \"%s\"]\n"
                  "    [v3 vector3r \"%s\"]\n}\n" % (p.name, p.material, v3(p.v1), v3(p.v2), v3(p.v3)))
            elif isinstance(p, Rectangle):
                w("primitive {\n    [type string \"rectangle\"]\n    [name string \"%s\"]\n"
                  "    [bsdf material \"%s\"]\n    [v1 vector3r \"%s\"]\n    [v2 vector3r \"%s\"]\n"
                  "    [v3 vector3r \"%s\"]\n}\n" % (p.name, p.material, v3(p.v1), v3(p.v2), v3(p.v3)))
            elif isinstance(p, Sphere):
                w("primitive {\n    [type string \"sphere\"]\n    [name string \"%s\"]\n"
                  "    [bsdf material \"%s\"]\n    [center vector3r \"%s\"]\n    [radius real \"%.9g\"]\n}\n"
                  % (p.name, p.material, v3(p.center), p.radius))
            elif sidecar is not None and p.positions.shape[0] >= sidecar[2]:
                import os
                base, stem, _ = sidecar
                w("primitive {\n    [type string \"triangle-mesh\"]\n    [name string \"%s\"]\n"
                  "    [bsdf material \"%s\"]\n" % (p.name, p.material))
                for key, arr in (("positions", p.positions), ("normals", p.normals), ("uvws", p.uvws)):
                    if arr is None:
                        continue
                    fn = "%s.%s.%s.f32" % (stem, p.name, key)
                    np.ascontiguousarray(arr, dtype="<f4").tofile(os.path.join(base, fn))
                    w("    [%s-file string \"%s\"]\n" % (key, fn))
                w("}\n")
            else:
                pos = p.positions.reshape(-1, 3)
                w("primitive {\n    [type string \"triangle-mesh\"]\n    [name string \"%s\"]\n"
                  "    [bsdf material \"%s\"]\n" % (p.name, p.material))
                w("    [positions vector3r-array \"%s\"]\n" % ", ".join(v3(v) for v in pos))
                if p.normals is not None:
                    w("    [normals vector3r-array \"%s\"]\n"
                      % ", ".join(v3(v) for v in p.normals.reshape(-1, 3)))
                if p.uvws is not None:
                    w("    [uvws vector3r-array \"%s\"]\n"
                      % ", ".join(v3(v) for v in p.uvws.reshape(-1, 3)))
                w("}\n")
        for lt in self.lights:
            w("light {\n    [type string \"area\"]\n    [primitive primitive \"%s\"]\n"
              "    [color rgb \"%s\"]\n    [watt real \"%.9g\"]\n"
              "    [is-back-face-emit bool \"%s\"]\n}\n"
              % (lt.primitive, v3(lt.color), lt.watt, "true" if lt.back_face_emit else "false"))
        return "".join(out)


# --------------------------------------------------------------------------
# geometry helpers
# --------------------------------------------------------------------------

def _box_triangles(size, center_xz, angle_deg, y0=0.0) -> np.ndarray:
    """12 outward-wound triangles of an axis-aligned box rotated about +y."""
    sx, sy, sz = size
    hx, hz = sx * 0.5, sz * 0.5
    corners = np.array([[x, y, z] for y in (y0, y0 + sy) for z in (-hz, hz) for x in (-hx, hx)],
                       dtype=np.float64)
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    rot = np.array([[ca, 0.0, sa], [0.0, 1.0, 0.0], [-sa, 0.0, ca]])
    corners = corners @ rot.T
    corners[:, 0] += center_xz[0]
    corners[:, 2] += center_xz[1]
    # corner index = x + 2*z + 4*y
    quads = [(0, 1, 3, 2),  # bottom (y0)
             (4, 6, 7, 5),  # top
             (0, 4, 5, 1),  # z = -hz
             (2, 3, 7, 6),  # z = +hz
             (0, 2, 6, 4),  # x = -hx
             (1, 5, 7, 3)]  # x = +hx
    tris = []
    for a0, a1, a2, a3 in quads:
        tris.append([corners[a0], corners[a1], corners[a2]])
        tris.append([corners[a0], corners[a2], corners[a3]])
    return np.asarray(tris, dtype=np.float32)


def _quad_light_watt(emission, area) -> float:
    return float(sum(emission)) * float(area) * math.pi


def cornell_box(width: int = 256, height: int = 256, spp: int = 16, max_depth: int = 6) -> SceneSpec:
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(278.0, 278.0, -800.0), cam_direction=(0.0, 0.0, 1.0),
                  cam_up=(0.0, 1.0, 0.0), fov=40.0)
    s.materials = [Material("white", LAMBERT, albedo=(0.725, 0.71, 0.68)),
                   Material("red", LAMBERT, albedo=(0.63, 0.065, 0.05)),
                   Material("green", LAMBERT, albedo=(0.14, 0.45, 0.091))]
    L = 556.0
    s.primitives = [
        Rectangle("floor", "white", (L, 0, 0), (0, 0, 0), (0, 0, L)),
        Rectangle("ceiling", "white", (0, L, 0), (L, L, 0), (L, L, L)),
        Rectangle("back", "white", (0, 0, L), (L, 0, L), (L, L, L)),
        Rectangle("left", "green", (0, 0, 0), (0, 0, L), (0, L, L)),
        Rectangle("right", "red", (L, 0, L), (L, 0, 0), (L, L, 0)),
        TriangleMesh("shortBox", "white", _box_triangles((165, 165, 165), (185.5, 169.0), -18.0)),
        TriangleMesh("tallBox", "white", _box_triangles((165, 330, 165), (368.5, 351.0), 15.0)),
        Rectangle("light", "white", (343.0, 555.0, 225.5), (213.0, 555.0, 225.5), (213.0, 555.0, 330.5)),
    ]
    emission = (17.0, 12.0, 4.0)
    s.lights = [AreaLight("light", emission, _quad_light_watt(emission, 130.0 * 105.0))]
    return s


def icosphere(subdivision: int) -> np.ndarray:
    """Unit icosphere triangles, (20 * 4**subdivision, 3, 3) float64."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    v = np.asarray(verts, dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    tris = v[np.asarray(faces)]
    for _ in range(subdivision):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab = a + b
        bc = b + c
        ca = c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                         np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    return tris


def _value_noise(p: np.ndarray, lattice: np.ndarray, freq: float) -> np.ndarray:
    """Trilinear smoothstep value noise in [-1, 1] from a periodic lattice."""
    n = lattice.shape[0]
    q = p * freq
    i0 = np.floor(q).astype(np.int64)
    f = q - i0
    f = f * f * (3.0 - 2.0 * f)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = ((f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1])
                     * (f[:, 2] if dz else 1 - f[:, 2]))
                ix = (i0[:, 0] + dx) % n
                iy = (i0[:, 1] + dy) % n
                iz = (i0[:, 2] + dz) % n
                out += w * lattice[ix, iy, iz]
    return out


def icosphere_field(n_spheres: int = 200, subdivision: int = 4, n_lights: int = 8, seed: int = 2,
                    width: int = 1920, height: int = 1080, spp: int = 64, max_depth: int = 12,
                    dielectric: str = ROUGH_DIELECTRIC, box: float = 100.0,
                    radius_range=(3.0, 8.0), displacement: float = 0.10, palette: int = 0) -> SceneSpec:
    """Displaced icospheres with centres uniform in a ``box``^3 cube over a
    2-triangle ground plane; materials drawn uniformly from Lambert
    (albedo U[0.05,0.9]^3), GGX conductor (roughness U[0.05,0.6], F0
    U[0.5,1]^3) and dielectric (IOR U[1.3,1.7]); quad lights with emission
    log-uniform in [1, 50].

    palette > 0: the spheres share `palette` GGX materials (conductors and
    dielectrics in turn) and palette / 2 Lambert materials, drawn from their
    own seeded stream, instead of one material each; a sphere keeps its kind
    (Lambert or GGX) and its geometry, so the scene differs only in its
    material table (a fixed set of roughness parameters for the adjoint)."""
    rng = np.random.default_rng(seed)
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.5 * box, 0.75 * box, -0.95 * box),
                  cam_direction=(0.0, -0.35, 1.0), cam_up=(0.0, 1.0, 0.0), fov=55.0)
    s.materials.append(Material("ground", LAMBERT, albedo=(0.5, 0.5, 0.5)))
    g = 2.0 * box
    y0 = -1.0
    ground = np.array([[[-g, y0, -g], [g, y0, g], [g, y0, -g]],
                       [[-g, y0, -g], [-g, y0, g], [g, y0, g]]], dtype=np.float32)
    s.primitives.append(TriangleMesh("ground", "ground", ground))
    unit = icosphere(subdivision)
    flat = unit.reshape(-1, 3)
    kinds = []
    for i in range(n_spheres):
        kind = int(rng.integers(0, 3))
        kinds.append(kind)
        name = "m%d" % i
        if kind == 0:
            s.materials.append(Material(name, LAMBERT, albedo=tuple(rng.uniform(0.05, 0.9, 3))))
        elif kind == 1:
            s.materials.append(Material(name, CONDUCTOR, roughness=float(rng.uniform(0.05, 0.6)),
                                        f0=tuple(rng.uniform(0.5, 1.0, 3))))
        else:
            s.materials.append(Material(name, dielectric, albedo=(1.0, 1.0, 1.0),
                                        roughness=float(rng.uniform(0.05, 0.3)),
                                        ior_inner=float(rng.uniform(1.3, 1.7))))
        centre = rng.uniform(0.0, box, 3)
        radius = float(rng.uniform(*radius_range))
        lattice = rng.uniform(-1.0, 1.0, (8, 8, 8))
        disp = 1.0 + displacement * _value_noise(flat + 1.0, lattice, 1.7)
        pos = (flat * (radius * disp)[:, None] + centre).astype(np.float32).reshape(-1, 3, 3)
        s.primitives.append(TriangleMesh("sphere%d" % i, name, pos))
    if palette > 0:
        prng = np.random.default_rng(seed + 7919)
        ggx, lam = [], []
        for k in range(palette):
            if k % 2 == 0:
                ggx.append(Material("ggx%d" % k, CONDUCTOR, roughness=float(prng.uniform(0.05, 0.6)),
                                    f0=tuple(prng.uniform(0.5, 1.0, 3))))
            else:
                ggx.append(Material("ggx%d" % k, dielectric, albedo=(1.0, 1.0, 1.0),
                                    roughness=float(prng.uniform(0.05, 0.3)), ior_inner=float(prng.uniform(1.3, 1.7))))
        for k in range(max(1, palette // 2)):
            lam.append(Material("lambert%d" % k, LAMBERT, albedo=tuple(prng.uniform(0.05, 0.9, 3))))
        s.materials = [s.materials[0]] + ggx + lam
        pick = prng.integers(0, 1 << 30, n_spheres)
        for i, kind in enumerate(kinds):
            s.primitives[1 + i].material = lam[pick[i] % len(lam)].name if kind == 0 else ggx[pick[i] % len(ggx)].name
    s.materials.append(Material("lightBase", LAMBERT, albedo=(0.5, 0.5, 0.5)))
    side = 0.15 * box
    for j in range(n_lights):
        cx, cz = rng.uniform(0.0, box, 2)
        y = 1.3 * box
        e = float(math.exp(rng.uniform(math.log(1.0), math.log(50.0))))
        name = "quadLight%d" % j
        # v1 - v2 = +x edge, v3 - v2 = +z edge: normal (+x) x (+z) = -y (down)
        s.primitives.append(Rectangle(name, "lightBase", (cx + side / 2, y, cz - side / 2),
                                      (cx - side / 2, y, cz - side / 2), (cx - side / 2, y, cz + side / 2)))
        s.lights.append(AreaLight(name, (e, e, e), _quad_light_watt((e, e, e), side * side)))
    return s


def feature_scene(width: int = 48, height: int = 40, spp: int = 16, max_depth: int = 8, seed: int = 11,
                  dielectric: str = GLASS) -> SceneSpec:
    """Small scene touching every primitive / light / BSDF path of the
    estimator: rectangle walls, single-triangle area lights (one two-sided),
    a smooth-normal icosphere mesh with per-vertex uvws, flat icospheres in
    Lambert, GGX conductor and dielectric, a rectangle light."""
    rng = np.random.default_rng(seed)
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.0, 6.0, -22.0), cam_direction=(0.0, -0.2, 1.0),
                  cam_up=(0.0, 1.0, 0.0), fov=50.0)
    s.materials = [Material("floor", LAMBERT, albedo=(0.6, 0.6, 0.55)),
                   Material("wall", LAMBERT, albedo=(0.3, 0.5, 0.7)),
                   Material("gold", CONDUCTOR, roughness=0.25, f0=(1.0, 0.78, 0.34)),
                   Material("steel", CONDUCTOR, roughness=0.05, f0=(0.56, 0.57, 0.58)),
                   Material("glass", dielectric, albedo=(1.0, 1.0, 1.0), roughness=0.15, ior_inner=1.5),
                   Material("clay", LAMBERT, albedo=(0.8, 0.35, 0.2)),
                   Material("emitterBase", LAMBERT, albedo=(0.2, 0.2, 0.2))]
    s.primitives.append(Rectangle("floor", "floor", (15, 0, -15), (-15, 0, -15), (-15, 0, 15)))
    s.primitives.append(Rectangle("back", "wall", (-15, 0, 12), (15, 0, 12), (15, 20, 12)))
    unit = icosphere(2)
    smooth = (unit / np.linalg.norm(unit, axis=2, keepdims=True)).astype(np.float32)
    uv = np.zeros_like(smooth)
    uv[..., 0] = 0.5 + np.arctan2(smooth[..., 0], smooth[..., 2]) / (2 * math.pi)
    uv[..., 1] = 0.5 + np.arcsin(np.clip(smooth[..., 1], -1, 1)) / math.pi
    s.primitives.append(TriangleMesh("smooth", "clay", (unit * 3.0 + [-6.0, 3.0, 2.0]).astype(np.float32),
                                     normals=smooth, uvws=uv.astype(np.float32)))
    for j, (mname, c, r) in enumerate([("gold", (0.0, 2.5, 0.0), 2.5), ("steel", (6.0, 2.0, -2.0), 2.0),
                                       ("glass", (1.5, 1.5, -6.0), 1.5)]):
        s.primitives.append(TriangleMesh("ball%d" % j, mname, (unit * r + c).astype(np.float32)))
    s.primitives.append(Triangle("triLight", "emitterBase", (-4, 12, -2), (4, 12, -2), (0, 12, 4)))
    s.primitives.append(Triangle("sideLight", "emitterBase", (12, 2, -4), (12, 8, 0), (12, 2, 4)))
    s.primitives.append(Rectangle("quadLight", "emitterBase", (3, 10, 6), (-3, 10, 6), (-3, 10, 9)))
    s.lights = [AreaLight("triLight", (10.0, 9.0, 8.0), 10.0 * 1.0),
                AreaLight("sideLight", (2.0, 4.0, 8.0), 600.0, back_face_emit=True),
                AreaLight("quadLight", (6.0, 6.0, 5.0), _quad_light_watt((6.0, 6.0, 5.0), 18.0))]
    # watt of the triangle light chosen so its radiance is ~(17, 15, 13)
    s.lights[0].watt = float(sum((10.0, 9.0, 8.0))) * 24.0 * math.pi * 1.7
    return s


def _smooth_texture(rng, size: int, lo: float = 0.2, hi: float = 0.8) -> np.ndarray:
    """Seeded smooth RGB pattern in [lo, hi] (sum of a few random sinusoids)."""
    y, x = np.mgrid[0:size, 0:size].astype(np.float64) / size
    img = np.zeros((size, size, 3))
    for c in range(3):
        acc = np.zeros((size, size))
        for _ in range(4):
            fx, fy = rng.integers(1, 6, 2)
            ph = rng.uniform(0, 2 * math.pi, 2)
            acc += np.sin(2 * math.pi * fx * x + ph[0]) * np.cos(2 * math.pi * fy * y + ph[1])
        acc = (acc - acc.min()) / max(acc.max() - acc.min(), 1e-9)
        img[..., c] = lo + (hi - lo) * acc
    return img.astype(np.float32)


def diff_scene(width: int = 512, height: int = 512, spp: int = 32, max_depth: int = 6, seed: int = 4,
               n_spheres: int = 20, subdivision: int = 4, tex_size: int = 256, n_conductors: int = 8,
               n_lights: int = 4) -> SceneSpec:
    """Differentiable-rendering scene: `n_spheres` displaced icospheres (20 x
    subdivision 4 = 102,400 triangles) over a ground plane; the Lambert
    spheres and the ground share one RGB float albedo texture with uniform
    (spherical / planar) uvs, `n_conductors` spheres each have their own GGX
    conductor material (one roughness parameter each), and `n_lights` quad
    lights carry the emitter-radiance parameters."""
    rng = np.random.default_rng(seed)
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.0, 9.0, -26.0), cam_direction=(0.0, -0.35, 1.0), cam_up=(0.0, 1.0, 0.0),
                  fov=50.0)
    s.textures.append(ImageTexture("albedoTex", _smooth_texture(rng, tex_size)))
    s.materials.append(Material("texLambert", LAMBERT, albedo_texture="albedoTex"))
    for k in range(n_conductors):
        s.materials.append(Material("metal%d" % k, CONDUCTOR, roughness=float(rng.uniform(0.2, 0.5)),
                                    f0=tuple(rng.uniform(0.6, 0.95, 3))))
    s.materials.append(Material("lightBase", LAMBERT, albedo=(0.3, 0.3, 0.3)))
    g = 20.0
    ground = np.array([[[-g, 0, -g], [g, 0, g], [g, 0, -g]], [[-g, 0, -g], [-g, 0, g], [g, 0, g]]], np.float32)
    guv = np.zeros_like(ground)
    guv[..., 0] = (ground[..., 0] + g) / (2 * g)
    guv[..., 1] = (ground[..., 2] + g) / (2 * g)
    s.primitives.append(TriangleMesh("ground", "texLambert", ground, uvws=guv))
    unit = icosphere(subdivision)
    flat = unit.reshape(-1, 3)
    for i in range(n_spheres):
        r = float(rng.uniform(1.0, 2.2))
        c = np.array([rng.uniform(-9, 9), r, rng.uniform(-6, 9)])
        lattice = rng.uniform(-1.0, 1.0, (8, 8, 8))
        disp = 1.0 + 0.1 * _value_noise(flat + 1.0, lattice, 1.7)
        pos = (flat * (r * disp)[:, None] + c).astype(np.float32).reshape(-1, 3, 3)
        if i < n_conductors:
            s.primitives.append(TriangleMesh("ball%d" % i, "metal%d" % i, pos))
        else:
            n = unit / np.linalg.norm(unit, axis=2, keepdims=True)
            uv = np.zeros_like(unit)
            uv[..., 0] = 0.5 + np.arctan2(n[..., 0], n[..., 2]) / (2 * math.pi)
            uv[..., 1] = 0.5 + np.arcsin(np.clip(n[..., 1], -1, 1)) / math.pi
            s.primitives.append(TriangleMesh("ball%d" % i, "texLambert", pos, uvws=uv.astype(np.float32)))
    for j in range(n_lights):
        cx, cz = rng.uniform(-8, 8, 2)
        e = float(rng.uniform(4.0, 12.0))
        col = tuple(float(x) for x in e * rng.uniform(0.6, 1.0, 3))
        name = "lamp%d" % j
        h = 3.0
        s.primitives.append(Rectangle(name, "lightBase", (cx + h, 14.0, cz - h), (cx - h, 14.0, cz - h),
                                      (cx - h, 14.0, cz + h)))
        s.lights.append(AreaLight(name, col, _quad_light_watt(col, (2 * h) ** 2)))
    return s


def texture_scene(width: int = 48, height: int = 40, spp: int = 16, max_depth: int = 6, seed: int = 17,
                  tex_w: int = 16, tex_h: int = 12) -> SceneSpec:
    """Image-texture scene: a floor and a back wall (two-triangle meshes) and
    a smooth icosphere share one RGB albedo texture of `tex_w` x `tex_h`
    distinct seeded texels, looked up nearest with repeat wrap.  The floor's
    uvs run from -1.5 to 2.25 and from -0.75 to 2.5 (negative coordinates
    and several wraps), the wall's from 0 to 3 and 0 to 2 (texel borders on
    its edges), the sphere's are spherical; a plain Lambert sphere and a
    rectangle light overhead."""
    rng = np.random.default_rng(seed)
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.0, 7.0, -20.0), cam_direction=(0.0, -0.3, 1.0),
                  cam_up=(0.0, 1.0, 0.0), fov=55.0)
    s.textures.append(ImageTexture("albedoTex", rng.uniform(0.05, 0.95, (tex_h, tex_w, 3)).astype(np.float32)))
    s.materials = [Material("tex", LAMBERT, albedo_texture="albedoTex"),
                   Material("clay", LAMBERT, albedo=(0.7, 0.4, 0.3)),
                   Material("emitterBase", LAMBERT, albedo=(0.2, 0.2, 0.2))]
    f = 14.0
    floor = np.array([[[-f, 0, -f], [f, 0, f], [f, 0, -f]], [[-f, 0, -f], [-f, 0, f], [f, 0, f]]], np.float32)
    fuv = np.zeros_like(floor)
    fuv[..., 0] = -1.5 + (floor[..., 0] + f) / (2 * f) * 3.75
    fuv[..., 1] = -0.75 + (floor[..., 2] + f) / (2 * f) * 3.25
    s.primitives.append(TriangleMesh("floor", "tex", floor, uvws=fuv.astype(np.float32)))
    wall = np.array([[[-f, 0, 10], [f, 16, 10], [f, 0, 10]], [[-f, 0, 10], [-f, 16, 10], [f, 16, 10]]], np.float32)
    wuv = np.zeros_like(wall)
    wuv[..., 0] = (wall[..., 0] + f) / (2 * f) * 3.0
    wuv[..., 1] = wall[..., 1] / 16.0 * 2.0
    s.primitives.append(TriangleMesh("wall", "tex", wall, uvws=wuv.astype(np.float32)))
    unit = icosphere(2)
    n = unit / np.linalg.norm(unit, axis=2, keepdims=True)
    uv = np.zeros_like(unit)
    uv[..., 0] = 0.5 + np.arctan2(n[..., 0], n[..., 2]) / (2 * math.pi)
    uv[..., 1] = 0.5 + np.arcsin(np.clip(n[..., 1], -1, 1)) / math.pi
    s.primitives.append(TriangleMesh("ball", "tex", (unit * 3.0 + [-4.0, 3.0, 2.0]).astype(np.float32),
                                     uvws=uv.astype(np.float32)))
    s.primitives.append(TriangleMesh("plain", "clay", (unit * 2.0 + [5.0, 2.0, -1.0]).astype(np.float32)))
    s.primitives.append(Rectangle("light", "emitterBase", (3, 12, -2), (-3, 12, -2), (-3, 12, 4)))
    emission = (9.0, 8.0, 7.0)
    s.lights = [AreaLight("light", emission, _quad_light_watt(emission, 36.0))]
    return s


def roughness_scene(width: int = 64, height: int = 48, spp: int = 64, max_depth: int = 3) -> SceneSpec:
    """Close-up of three GGX spheres for finite-difference checks of the
    roughness gradient: two conductors (roughness 0.55 and 0.5) and a rough
    dielectric (roughness 0.3, IOR 1.5) on a Lambert floor under two quad
    lights, framed so that most pixels see a GGX surface (pixels whose paths
    never meet one add nothing to either the gradient or its noise)."""
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.0, 2.6, -8.5), cam_direction=(0.0, -0.18, 1.0), cam_up=(0.0, 1.0, 0.0),
                  fov=40.0)
    s.materials = [Material("floor", LAMBERT, albedo=(0.55, 0.5, 0.45)),
                   Material("gold", CONDUCTOR, roughness=0.55, f0=(1.0, 0.78, 0.34)),
                   Material("steel", CONDUCTOR, roughness=0.5, f0=(0.6, 0.6, 0.62)),
                   Material("frost", ROUGH_DIELECTRIC, albedo=(1.0, 1.0, 1.0), roughness=0.3, ior_inner=1.5),
                   Material("emitterBase", LAMBERT, albedo=(0.2, 0.2, 0.2))]
    f = 12.0
    s.primitives.append(TriangleMesh("floor", "floor", np.array(
        [[[-f, 0, -f], [f, 0, f], [f, 0, -f]], [[-f, 0, -f], [-f, 0, f], [f, 0, f]]], np.float32)))
    unit = icosphere(3)
    for name, mat, cx in (("ballA", "gold", -2.6), ("ballB", "steel", 0.0), ("ballC", "frost", 2.6)):
        s.primitives.append(TriangleMesh(name, mat, (unit * 1.2 + [cx, 1.2, 0.0]).astype(np.float32)))
    s.primitives.append(Rectangle("lampA", "emitterBase", (2.0, 6.0, -3.0), (-2.0, 6.0, -3.0), (-2.0, 6.0, 1.0)))
    s.primitives.append(Rectangle("lampB", "emitterBase", (5.0, 4.0, 2.0), (4.0, 4.0, 2.0), (4.0, 4.0, 3.0)))
    s.lights = [AreaLight("lampA", (6.0, 6.0, 5.5), _quad_light_watt((6.0, 6.0, 5.5), 16.0)),
                AreaLight("lampB", (20.0, 14.0, 8.0), _quad_light_watt((20.0, 14.0, 8.0), 1.0))]
    return s


def sphere_box(width: int = 64, height: int = 48, spp: int = 16, max_depth: int = 8) -> SceneSpec:
    """Open-front box of rectangles with analytic spheres in every non-GGX
    material the reference has besides Lambert: plastic (Lambert + Phong mix),
    Phong, mirror with a conductor and with a dielectric Fresnel term, a
    smooth conductor, and glass; one rectangular ceiling light."""
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth, cam_position=(280.0, 270.0, 780.0),
                  cam_direction=(0.0, 0.0, -1.0), cam_up=(0.0, 1.0, 0.0), fov=50.0)
    s.materials = [
        Material("white", LAMBERT, albedo=(0.72, 0.72, 0.70)),
        Material("red", LAMBERT, albedo=(0.70, 0.28, 0.25)),
        Material("blue", LAMBERT, albedo=(0.25, 0.30, 0.72)),
        Material("plastic", PLASTIC, albedo=(0.70, 0.55, 0.05), exponent=16.0, diffuse_ratio=0.8),
        Material("phong", PHONG, exponent=24.0),
        Material("chrome", MIRROR, albedo=(0.95, 0.95, 0.95), fresnel="conductor", f0=(0.9, 0.85, 0.8)),
        Material("glassMirror", MIRROR, albedo=(1.0, 1.0, 1.0), fresnel="dielectric", ior_outer=1.0,
                 ior_inner=1.6),
        Material("steel", CONDUCTOR, roughness=0.0, f0=(1.0, 1.0, 1.0)),
        Material("glass", GLASS, albedo=(1.0, 1.0, 1.0), ior_outer=1.0, ior_inner=1.5),
    ]
    W, H, D = 560.0, 550.0, -650.0
    s.primitives = [
        Rectangle("left", "red", (-80.0, 0.0, D), (-80.0, 0.0, 0.0), (-80.0, H, 0.0)),
        Rectangle("right", "blue", (640.0, 0.0, 0.0), (640.0, 0.0, D), (640.0, H, D)),
        Rectangle("top", "white", (645.0, H, 0.0), (-85.0, H, 0.0), (-85.0, H, D)),
        Rectangle("back", "white", (-85.0, H, D), (645.0, H, D), (645.0, 0.0, D)),
        Rectangle("floor", "white", (645.0, 0.0, 0.0), (-85.0, 0.0, 0.0), (-85.0, 0.0, D)),
        Sphere("plasticBall", "plastic", (100.0, 100.0, -360.0), 100.0),
        Sphere("steelBall", "steel", (420.0, 110.0, -220.0), 110.0),
        Sphere("phongBall", "phong", (300.0, 60.0, -470.0), 60.0),
        Sphere("chromeBall", "chrome", (520.0, 300.0, -520.0), 70.0),
        Sphere("mirrorBall", "glassMirror", (60.0, 330.0, -560.0), 55.0),
        Sphere("glassBall", "glass", (250.0, 260.0, -300.0), 45.0),
        Rectangle("light", "white", (370.0, H - 10.0, -170.0), (370.0, H - 10.0, -330.0), (185.0, H - 10.0, -330.0)),
    ]
    s.lights = [AreaLight("light", (1.0, 1.0, 1.0), 5.0e6)]
    return s


def coplanar_scene(width: int = 40, height: int = 30, spp: int = 16, max_depth: int = 8) -> SceneSpec:
    """Coplanar, overlapping primitives - where the reference's closest hit
    is decided by the order of its BVH traversal: quad lights of different
    emission lying in the ceiling's own plane and overlapping one another
    (one inside another, two identical), and rectangles and triangle meshes
    of different albedos overlapping on the floor's plane, seen directly and
    in a glossy wall."""
    H, W = 10.0, 10.0
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth,
                  cam_position=(0.0, 4.5, -9.5), cam_direction=(0.0, 0.2, 1.0), cam_up=(0.0, 1.0, 0.0), fov=85.0)
    s.materials = [Material("white", LAMBERT, albedo=(0.72, 0.71, 0.68)),
                   Material("grey", LAMBERT, albedo=(0.45, 0.45, 0.45)),
                   Material("red", LAMBERT, albedo=(0.7, 0.1, 0.08)),
                   Material("green", LAMBERT, albedo=(0.12, 0.6, 0.1)),
                   Material("blue", LAMBERT, albedo=(0.1, 0.15, 0.7)),
                   Material("yellow", LAMBERT, albedo=(0.75, 0.7, 0.1)),
                   Material("steel", CONDUCTOR, roughness=0.08, f0=(0.9, 0.9, 0.92)),
                   Material("lightBase", LAMBERT, albedo=(0.3, 0.3, 0.3))]

    def rect_xz(name, mat, x0, x1, z0, z1, y):
        # v1 - v2 = +x edge, v3 - v2 = +z edge: the normal faces -y
        return Rectangle(name, mat, (x1, y, z0), (x0, y, z0), (x0, y, z1))

    def quad_mesh(name, mat, x0, x1, z0, z1, y):
        a, b, c, d = (x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z1)
        return TriangleMesh(name, mat, np.array([[a, b, c], [a, c, d]], np.float32))

    s.primitives = [
        rect_xz("ceiling", "white", -W, W, -W, W, H),
        rect_xz("floor", "grey", -W, W, -W, W, 0.0),
        Rectangle("back", "white", (-W, 0, W), (W, 0, W), (W, H, W)),
        Rectangle("left", "grey", (-W, 0, -W), (-W, 0, W), (-W, H, W)),
        Rectangle("right", "steel", (W, 0, W), (W, 0, -W), (W, H, -W)),
        rect_xz("redTile", "red", -6.0, 0.0, -2.0, 6.0, 0.0),
        rect_xz("greenTile", "green", -3.0, 3.0, 0.0, 8.0, 0.0),
        quad_mesh("blueTile", "blue", 1.0, 7.0, -4.0, 2.0, 0.0),
        quad_mesh("yellowTile", "yellow", 4.0, 9.0, -1.0, 5.0, 0.0),
    ]
    lights = [("light0", -6.0, -1.0, 0.0, 5.0, (8.0, 8.0, 8.0)),
              ("light1", -4.0, 1.0, 2.0, 7.0, (2.0, 5.0, 10.0)),
              ("light2", 2.0, 7.0, 1.0, 6.0, (12.0, 6.0, 2.0)),
              ("light3", 2.0, 7.0, 1.0, 6.0, (1.0, 1.0, 1.0)),  # light2's own rectangle
              ("light4", 3.0, 5.0, 2.0, 4.0, (4.0, 12.0, 4.0))]  # inside light2
    for name, x0, x1, z0, z1, e in lights:
        s.primitives.append(rect_xz(name, "lightBase", x0, x1, z0, z1, H))
        s.lights.append(AreaLight(name, e, _quad_light_watt(e, (x1 - x0) * (z1 - z0))))
    return s


def power_field(width: int = 48, height: int = 36, spp: int = 16, max_depth: int = 8, seed: int = 21) -> SceneSpec:
    """Small icosphere field (glass, conductors, Lambert) under 6 quad lights
    of log-uniform emission, lights picked by the power light cluster."""
    s = icosphere_field(n_spheres=10, subdivision=2, n_lights=6, seed=seed, width=width, height=height, spp=spp,
                        max_depth=max_depth, dielectric=GLASS, box=30.0, radius_range=(2.0, 6.0))
    s.light_cluster = "power"
    return s


def batch_scenes(count: int = 64, seed: int = 3, tri_range=(10_000, 2_000_000)) -> list:
    """The batched configuration: `count` icosphere fields with triangle
    counts log-uniform in `tri_range` (subdivision 4 spheres of 5,120
    triangles, or subdivision 3 of 1,280 below 51,200), each with its own
    resolution from {128, 256, 512, 1024}^2, spp from {4, 16, 64, 256} and
    max depth from {4, 8, 16}."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        tris = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
        sub = 4 if tris >= 51_200 else 3
        n = max(1, int(round(tris / (20 * 4 ** sub))))
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = int(rng.choice([4, 16, 64, 256]))
        depth = int(rng.choice([4, 8, 16]))
        out.append(icosphere_field(n_spheres=n, subdivision=sub, n_lights=8, seed=1000 + i, width=res, height=res,
                                   spp=spp, max_depth=depth, box=100.0 * (n / 200.0) ** (1 / 3)))
    return out


def lognormal_sky(width: int = 2048, height: int = 1024, sigma: float = 1.5, seed: int = 5) -> np.ndarray:
    """Procedural HDR environment map: smooth log-normal luminance field
    (log-luminance ~ N(0, sigma^2), spatially correlated) with a warm/cool tint."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:height, 0:width].astype(np.float64)
    u, v = x / width, y / height
    field = np.zeros((height, width))
    for k in range(12):
        fu, fv = rng.integers(1, 8), rng.integers(1, 5)
        ph = rng.uniform(0, 2 * math.pi, 2)
        field += np.sin(2 * math.pi * fu * u + ph[0]) * np.sin(math.pi * fv * v + ph[1])
    field = (field - field.mean()) / max(field.std(), 1e-9) * sigma
    lum = np.exp(field)
    tint = np.stack([1.0 + 0.2 * v, np.ones_like(v), 1.2 - 0.3 * v], -1)
    return (lum[..., None] * tint).astype(np.float32)


def env_field(n_spheres: int = 4000, subdivision: int = 4, n_lights: int = 64, width: int = 3840, height: int = 2160,
              spp: int = 1024, max_depth: int = 32, seed: int = 7, sky: tuple = (2048, 1024),
              palette: int = 64) -> SceneSpec:
    """The stress configuration: displaced icospheres (4000 x subdivision 4
    = 20,480,000 triangles) over a ground plane, mixed Lambert / GGX
    conductor / GGX dielectric from a palette of `palette` GGX materials
    (the 64 roughness parameters of its adjoint) and palette / 2 Lambert
    ones, a log-normal HDR sky and quad lights (64 radiance parameters)."""
    s = icosphere_field(n_spheres=n_spheres, subdivision=subdivision, n_lights=n_lights, seed=seed, width=width,
                        height=height, spp=spp, max_depth=max_depth, box=100.0 * (n_spheres / 200.0) ** (1 / 3),
                        palette=palette)
    s.textures.append(ImageTexture("sky", lognormal_sky(sky[0], sky[1], 1.5, seed)))
    s.environment = "sky"
    return s


def furnace_scene(width: int = 32, height: int = 32, spp: int = 64, albedo: float = 0.5, sky: float = 1.0,
                  max_depth: int = 4) -> SceneSpec:
    """White-furnace check: a convex Lambert icosphere under a constant sky of
    radiance `sky`.  Light leaving the sphere never returns to it, so every
    pixel's expected radiance is exactly `albedo * sky` on the sphere and
    `sky` elsewhere."""
    s = SceneSpec(width=width, height=height, spp=spp, max_depth=max_depth, cam_position=(0.0, 0.0, -6.0),
                  cam_direction=(0.0, 0.0, 1.0), cam_up=(0.0, 1.0, 0.0), fov=40.0)
    s.materials = [Material("grey", LAMBERT, albedo=(albedo, albedo, albedo))]
    s.primitives = [TriangleMesh("ball", "grey", icosphere(3).astype(np.float32))]
    s.textures = [ImageTexture("sky", np.full((8, 16, 3), sky, np.float32))]
    s.environment = "sky"
    return s
