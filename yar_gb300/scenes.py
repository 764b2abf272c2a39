"""Seeded synthetic workloads (there are no published scenes for this path).

cornell_pbrt      - procedural Cornell box as a pbrt-v3 file: 5 wall quads, two
                    boxes rotated by seed-drawn angles in [0, 30] degrees
                    (34 triangles), Lambertian albedos U[0.2, 0.8] per channel,
                    one 0.25 x 0.25 quad light of radiance 17.
raycast_scene     - seeded fBm terrain heightfield (grid x grid cells, 2
                    triangles per cell, 6 octaves, amplitude 0.1) plus
                    icospheres (subdivision 4, 5120 triangles each) at uniform
                    random positions; one mesh per object, spheres placed by a
                    translation so the two-level transform path is exercised.
random_rays /
random_shadow_rays - origins uniform in the scene box, directions uniform on
                    the sphere; shadow rays have tmax = U[0,1] * |diagonal|.
"""
import math

import numpy as np

from . import native
from .scene import FlatScene, Mesh, make_object


# ---------------------------------------------------------------- icosphere
def icosphere(radius=1.0, level=4):
    """create_sphere_mesh (src/lib/tessellation.cpp:43-171): geodesic
    subdivision of an icosahedron with shared, deduplicated vertices."""
    f32 = np.float32
    t = f32((f32(1.0) + np.sqrt(f32(5.0))) / f32(2.0))
    s_inv = f32(f32(1.0) / np.sqrt(f32(1.0) + t * t))
    verts = [(t, 1, 0), (-t, 1, 0), (t, -1, 0), (-t, -1, 0), (1, 0, t), (1, 0, -t), (-1, 0, t), (-1, 0, -t),
             (0, t, 1), (0, -t, 1), (0, t, -1), (0, -t, -1)]
    verts = [np.array(v, f32) * s_inv for v in verts]
    idx = [0, 8, 4, 1, 10, 7, 2, 9, 11, 7, 3, 1, 0, 5, 10, 3, 9, 6, 3, 11, 9, 8, 6, 4, 2, 4, 9, 3, 7, 11,
           4, 2, 0, 9, 4, 6, 2, 11, 5, 0, 10, 8, 5, 0, 2, 10, 5, 7, 1, 6, 8, 1, 8, 10, 6, 1, 3, 11, 7, 5]

    def normalized(v):
        length = np.sqrt(f32(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]))
        return (v / length).astype(f32)

    for _ in range(level):
        new_verts, new_idx, lookup = [], [], {}

        def add(v):
            key = v.tobytes()
            if key not in lookup:
                lookup[key] = len(new_verts)
                new_verts.append(v)
            return lookup[key]

        for k in range(0, len(idx), 3):
            v0, v1, v2 = verts[idx[k]], verts[idx[k + 1]], verts[idx[k + 2]]
            v01, v12, v02 = normalized(v0 + v1), normalized(v1 + v2), normalized(v0 + v2)
            i0, i1, i2, i3, i4, i5 = add(v0), add(v1), add(v2), add(v01), add(v12), add(v02)
            new_idx += [i0, i3, i5, i3, i1, i4, i5, i4, i2, i3, i4, i5]
        verts, idx = new_verts, new_idx
    v = np.stack(verts).astype(np.float32) * np.float32(radius)
    return v.astype(np.float32), np.array(idx, np.int32).reshape(-1, 3)


# ---------------------------------------------------------------- terrain
def _value_noise(rng, freq, x, z):
    lattice = rng.random((freq + 2, freq + 2))
    fx, fz = x * freq, z * freq
    ix, iz = np.floor(fx).astype(np.int64), np.floor(fz).astype(np.int64)
    tx, tz = fx - ix, fz - iz
    sx, sz = tx * tx * (3 - 2 * tx), tz * tz * (3 - 2 * tz)
    a = lattice[ix, iz] * (1 - sx) + lattice[ix + 1, iz] * sx
    b = lattice[ix, iz + 1] * (1 - sx) + lattice[ix + 1, iz + 1] * sx
    return a * (1 - sz) + b * sz


def fbm_terrain(seed, grid=1024, octaves=6, amplitude=0.1, base_freq=4):
    rng = np.random.default_rng(seed)
    lin = np.linspace(0.0, 1.0, grid + 1)
    x, z = np.meshgrid(lin, lin, indexing="ij")
    h = np.zeros_like(x)
    norm = 0.0
    for k in range(octaves):
        w = 0.5 ** k
        h += w * (_value_noise(rng, base_freq * 2 ** k, x, z) - 0.5)
        norm += w
    h = amplitude * h / norm
    verts = np.stack([x, h, z], axis=-1).reshape(-1, 3).astype(np.float32)
    n = grid + 1
    i = np.arange(grid)
    ii, jj = np.meshgrid(i, i, indexing="ij")
    v00 = (ii * n + jj).reshape(-1)
    v10 = ((ii + 1) * n + jj).reshape(-1)
    v01 = (ii * n + jj + 1).reshape(-1)
    v11 = ((ii + 1) * n + jj + 1).reshape(-1)
    tris = np.empty((grid * grid * 2, 3), np.int32)
    tris[0::2] = np.stack([v00, v10, v11], axis=1)
    tris[1::2] = np.stack([v00, v11, v01], axis=1)
    return verts, tris


def raycast_scene(seed=1, grid=1024, spheres=64, level=4, build=True, threads=0):
    """The ray-cast benchmark scene: ~2.42M triangles at grid=1024, 64 spheres."""
    rng = np.random.default_rng(seed + 1000)
    s = FlatScene()
    tv, ti = fbm_terrain(seed, grid)
    s.meshes.append(Mesh(tv, ti))
    objects = [make_object(0)]
    lo = tv.min(axis=0)
    hi = tv.max(axis=0)
    sv, si = icosphere(1.0, level)
    for k in range(spheres):
        r = np.float32(rng.uniform(0.01, 0.04))
        c = rng.uniform([lo[0], lo[1], lo[2]], [hi[0], hi[1] + 0.1, hi[2]]).astype(np.float32)
        s.meshes.append(Mesh(sv * r, si))
        m = np.array([1, 0, 0, c[0], 0, 1, 0, c[1], 0, 0, 1, c[2]], np.float32)
        w = np.array([1, 0, 0, -c[0], 0, 1, 0, -c[1], 0, 0, 1, -c[2]], np.float32)
        objects.append(make_object(k + 1, m, w))
    s.objects = np.array(objects)
    if build:
        s.build_kdtrees(threads)
    return s


def scene_box(s):
    lo = s.scene_bounds[:3].astype(np.float64)
    hi = s.scene_bounds[3:].astype(np.float64)
    return lo, hi


def _uniform_sphere(rng, n):
    u0 = rng.random(n)
    u1 = rng.random(n)
    z = 1.0 - 2.0 * u0
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * math.pi * u1
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def random_rays(lo, hi, n, seed, tmax=np.inf):
    """(n, 8) float32 yar_ray records: origin, tmax, direction, pad."""
    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, size=(n, 3))
    rays[:, 3] = tmax
    rays[:, 4:7] = _uniform_sphere(rng, n)
    return rays


def random_shadow_rays(lo, hi, n, seed):
    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, size=(n, 3))
    rays[:, 4:7] = _uniform_sphere(rng, n)
    diag = float(np.linalg.norm(np.asarray(hi) - np.asarray(lo)))
    rays[:, 3] = rng.random(n) * diag
    return rays


# ---------------------------------------------------------------- Cornell box
def _quad(p0, p1, p2, p3):
    return np.array([p0, p1, p2, p3], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.int32)


def _box(center, size, angle_deg):
    cx, cz = center[0], center[2]
    sx, sy, sz = size
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)
    corners = []
    for y in (0.0, sy):
        for (dx, dz) in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            x = dx * sx / 2
            z = dz * sz / 2
            corners.append((cx + ca * x + sa * z, y, cz - sa * x + ca * z))
    v = np.array(corners, np.float32)
    idx = np.array([[0, 2, 1], [0, 3, 2],        # bottom
                    [4, 5, 6], [4, 6, 7],        # top
                    [0, 1, 5], [0, 5, 4],
                    [1, 2, 6], [1, 6, 5],
                    [2, 3, 7], [2, 7, 6],
                    [3, 0, 4], [3, 4, 7]], np.int32)
    return v, idx


def cornell_pbrt(seed=1, width=256, height=256, spp=16, maxdepth=8, light_radiance=17.0, box_materials=None,
                 upper_light=None, light_sources=(), mesh_lights=(), sphere_lights=(), named_materials=(),
                 integrator="path", light_samples=1, textures=(), wall_textures=None, pixel_filter='"box"',
                 extra_shapes=(), wall_materials=None):
    """pbrt-v3 text of the seeded Cornell box (34 triangles + a quad light).

    box_materials: None for matte boxes, or two pbrt material statements for
    the short and the tall box (e.g. metal and rough glass).
    upper_light: None, or (half size, height, radiance) of a second quad light
    above the ceiling, facing down; it reaches the room only through a ceiling
    that transmits (a perfect refractor set on the flattened scene).
    light_sources: pbrt LightSource statements added to the world (point,
    spot, distant).
    mesh_lights: (vertices, indices, normals or None, radiance) emitting
    triangle meshes that are not rectangles (the reference makes them
    triangle-mesh lights).
    sphere_lights: (center, radius, radiance) emitting pbrt spheres (sphere
    lights, shown by the reference's tessellated sphere).
    named_materials: pbrt MakeNamedMaterial statements (for "mix").
    integrator: "path" or "directlighting" (the reference's direct-lighting
    algorithm); light_samples: the quad light's "integer samples".
    textures: pbrt Texture statements; wall_textures: {wall index (0 floor,
    1 ceiling, 2 back, 3 left, 4 right): texture name} walls whose matte Kd is
    that texture, given uvs (0,0), (1,0), (1,1), (0,1) at their corners.
    wall_materials: {wall index: (material statement, extra shape parameters)}
    walls with that material, the same uvs and the extra parameters (e.g.
    per-vertex normals).
    extra_shapes: pbrt statements added after the room."""
    rng = np.random.default_rng(seed)
    k = int(math.ceil(math.sqrt(spp)))
    shapes = []
    walls = [
        _quad((-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)),      # floor
        _quad((-1, 2, -1), (-1, 2, 1), (1, 2, 1), (1, 2, -1)),      # ceiling
        _quad((-1, 0, -1), (-1, 2, -1), (1, 2, -1), (1, 0, -1)),    # back
        _quad((-1, 0, -1), (-1, 0, 1), (-1, 2, 1), (-1, 2, -1)),    # left
        _quad((1, 0, -1), (1, 2, -1), (1, 2, 1), (1, 0, 1)),        # right
    ]
    for v, i in walls:
        shapes.append((v, i, rng.uniform(0.2, 0.8, 3)))
    a0, a1 = rng.uniform(0.0, 30.0, 2)
    shapes.append(_box((0.35, 0, 0.3), (0.6, 0.6, 0.6), a0) + (rng.uniform(0.2, 0.8, 3),))
    shapes.append(_box((-0.35, 0, -0.35), (0.6, 1.2, 0.6), a1) + (rng.uniform(0.2, 0.8, 3),))
    h = 0.125
    light = _quad((-h, 1.98, -h), (h, 1.98, -h), (h, 1.98, h), (-h, 1.98, h))

    def fmt(a):
        return " ".join("%.9g" % x for x in np.asarray(a).reshape(-1))

    out = [
        "LookAt 0 1 3.5  0 1 0  0 1 0",
        'Camera "perspective" "float fov" [40]',
        'Film "image" "integer xresolution" [%d] "integer yresolution" [%d] "string filename" "cornell.exr"'
        % (width, height),
        'Sampler "stratified" "integer xsamples" [%d] "integer ysamples" [%d]' % (k, k),
        'Integrator "%s" "integer maxdepth" [%d]' % (integrator, maxdepth),
        'PixelFilter %s' % pixel_filter,
        "WorldBegin",
    ] + list(textures) + list(named_materials) + list(light_sources)
    wall_textures = wall_textures or {}
    for k, (v, i, albedo) in enumerate(shapes):
        material = 'Material "matte" "rgb Kd" [%s]' % fmt(albedo)
        shape = '  Shape "trianglemesh" "integer indices" [%s] "point P" [%s]' % (fmt(i), fmt(v))
        if box_materials is not None and k >= 5:
            material = box_materials[k - 5]
        if k in wall_textures:
            material = 'Material "matte" "texture Kd" "%s"' % wall_textures[k]
            shape += ' "float uv" [0 0 1 0 1 1 0 1]'
        if k in (wall_materials or {}):
            material, extra = wall_materials[k]
            shape += ' "float uv" [0 0 1 0 1 1 0 1]' + extra
        out += ["AttributeBegin",
                '  ' + material,
                shape,
                "AttributeEnd"]
    out += ["AttributeBegin",
            '  AreaLightSource "diffuse" "rgb L" [%s] "integer nsamples" [%d]' % (fmt([light_radiance] * 3),
                                                                              light_samples),
            '  Shape "trianglemesh" "integer indices" [%s] "point P" [%s]' % (fmt(light[1]), fmt(light[0])),
            "AttributeEnd"]
    for center, radius, radiance in sphere_lights:
        out += ["AttributeBegin",
                "  Translate %s" % fmt(center),
                '  AreaLightSource "diffuse" "rgb L" [%s]' % fmt(radiance),
                '  Shape "sphere" "float radius" [%s]' % fmt([radius]),
                "AttributeEnd"]
    for v, i, n, radiance in mesh_lights:
        shape = '  Shape "trianglemesh" "integer indices" [%s] "point P" [%s]' % (fmt(i), fmt(v))
        if n is not None:
            shape += ' "normal N" [%s]' % fmt(n)
        out += ["AttributeBegin",
                '  AreaLightSource "diffuse" "rgb L" [%s]' % fmt(radiance),
                shape,
                "AttributeEnd"]
    out += list(extra_shapes)
    if upper_light is not None:
        uh, uy, ul = upper_light
        v, i = _quad((-uh, uy, -uh), (uh, uy, -uh), (uh, uy, uh), (-uh, uy, uh))
        out += ["AttributeBegin",
                '  AreaLightSource "diffuse" "rgb L" [%s]' % fmt([ul] * 3),
                '  Shape "trianglemesh" "integer indices" [%s] "point P" [%s]' % (fmt(i), fmt(v)),
                "AttributeEnd"]
    out += ["WorldEnd", ""]
    return "\n".join(out)


DELTA_BOXES = ('Material "mirror" "rgb Kr" [0.9 0.85 0.8]',
               'Material "glass" "float index" [1.5] "rgb Kr" [0.95 0.95 0.95] "rgb Kt" [0.9 0.95 1]')

LAYERED_BOXES = ('Material "plastic" "rgb Kd" [0.6 0.25 0.1] "rgb Ks" [0.4 0.4 0.4] "float roughness" [0.15]',
                 'Material "substrate" "rgb Kd" [0.2 0.4 0.6] "rgb Ks" [0.06 0.05 0.04] '
                 '"float uroughness" [0.1] "float vroughness" [0.3]')

TRANSLUCENT_BOXES = ('Material "matte" "rgb Kd" [0.5 0.5 0.5]',
                     'Material "translucent" "rgb Kd" [0.3 0.35 0.4] "rgb Ks" [0.6 0.6 0.6] '
                     '"rgb reflect" [0.5 0.5 0.5] "rgb transmit" [0.5 0.45 0.4] "float roughness" [0.1]')


UBER_BOXES = ('Material "uber" "rgb Kd" [0.5 0.3 0.2] "rgb Ks" [0.3 0.3 0.3] "rgb Kr" [0.4 0.4 0.4] '
              '"float roughness" [0.15] "float index" [1.5]',
              'Material "uber" "rgb Kd" [0.2 0.4 0.5] "rgb Ks" [0.2 0.2 0.2] "rgb opacity" [0.6 0.7 0.8] '
              '"float uroughness" [0.1] "float vroughness" [0.3] "float index" [1.4]')


MIX_NAMED = ('MakeNamedMaterial "red" "string type" "matte" "rgb Kd" [0.7 0.2 0.15]',
             'MakeNamedMaterial "gold" "string type" "metal" "float roughness" [0.15] "rgb eta" [0.2 0.92 1.1] '
             '"rgb k" [3.9 2.45 2.14]',
             'MakeNamedMaterial "mirror" "string type" "mirror" "rgb Kr" [0.85 0.85 0.9]',
             'MakeNamedMaterial "plastic" "string type" "plastic" "rgb Kd" [0.2 0.5 0.3] "rgb Ks" [0.3 0.3 0.3] '
             '"float roughness" [0.1]')
MIX_BOXES = ('Material "mix" "string namedmaterial1" "red" "string namedmaterial2" "gold" "rgb amount" [0.3 0.4 0.5]',
             'Material "mix" "string namedmaterial1" "mirror" "string namedmaterial2" "plastic" "rgb amount" [0.4 0.4 0.4]')


ENVIRONMENT_CONSTANT = ('LightSource "infinite" "rgb L" [0.5 0.55 0.6]',)


def environment_map(width=64, height=32, seed=1):
    """A latitude-longitude sky: a vertical gradient, seeded noise and a small
    bright sun, as float32 (height, width, 3)."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height, dtype=np.float32) + 0.5) / height
    u = (np.arange(width, dtype=np.float32) + 0.5) / width
    sky = np.stack([0.3 + 0.5 * (1 - v), 0.4 + 0.5 * (1 - v), 0.6 + 0.6 * (1 - v)], axis=-1)[:, None, :]
    img = np.broadcast_to(sky, (height, width, 3)).copy()
    img *= (0.8 + 0.4 * rng.random((height, width, 1))).astype(np.float32)
    du = np.minimum(np.abs(u[None, :] - 0.3), 1 - np.abs(u[None, :] - 0.3))
    sun = np.exp(-((du / 0.03) ** 2 + ((v[:, None] - 0.35) / 0.05) ** 2))
    img += (40.0 * sun)[..., None] * np.array([1.0, 0.9, 0.7], np.float32)
    return img.astype(np.float32)


def texture_image(width=48, height=40, seed=3):
    """A linear RGB test texture of a size that is not a power of two (the
    reference upsamples it): 8 x 8 checks with seeded per-texel noise, as
    float32 (height, width, 3)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:height, 0:width]
    checks = (((x * 8) // width + (y * 8) // height) % 2).astype(np.float32)
    base = np.stack([0.15 + 0.7 * checks, 0.6 - 0.4 * checks, 0.3 + 0.2 * (x / width)], axis=-1)
    return (base * (0.85 + 0.3 * rng.random((height, width, 1)))).astype(np.float32)


def cutout_image(size=16, cells=4):
    """An alpha texture for the alpha test: cells x cells checks of 0 and 1
    (all three channels), size x size texels."""
    y, x = np.mgrid[0:size, 0:size]
    on = (((x * cells) // size + (y * cells) // size) % 2).astype(np.float32)
    return np.repeat(on[:, :, None], 3, axis=2)


def bump_image(size=32, seed=5):
    """A height map for bump mapping: concentric ripples plus seeded noise,
    heights in [0, 0.05] in all three channels, size x size texels."""
    rng = np.random.default_rng(seed)
    y, x = (np.mgrid[0:size, 0:size] + 0.5) / size
    r = np.hypot(x - 0.5, y - 0.5)
    h = 0.5 + 0.35 * np.sin(2 * math.pi * 5 * r) + 0.15 * rng.random((size, size))
    h = 0.05 * np.clip(h, 0.0, 1.0)
    return np.repeat(h[:, :, None], 3, axis=2).astype(np.float32)


def bump_panel(material, normals=True):
    """pbrt statements of a vertical quad across the front of the room (uvs
    repeat twice), with slightly splayed per-vertex normals when `normals`,
    so that the normal's uv derivatives take part in the bump."""
    v = [-0.7, 0.05, 0.5, 0.7, 0.05, 0.5, 0.7, 1.3, 0.5, -0.7, 1.3, 0.5]
    n = [-0.15, -0.1, 1, 0.15, -0.1, 1, 0.15, 0.1, 1, -0.15, 0.1, 1]
    shape = ('  Shape "trianglemesh" "integer indices" [0 1 2 0 2 3] "point P" [%s] "float uv" [0 0 2 0 2 2 0 2]'
             % " ".join("%g" % a for a in v))
    if normals:
        shape += ' "normal N" [%s]' % " ".join("%g" % a for a in n)
    return ("AttributeBegin", "  " + material, shape, "AttributeEnd")


def cutout_fence(texture="cutout", material='Material "matte" "rgb Kd" [0.8 0.7 0.3]'):
    """pbrt statements of a vertical quad across the room, between the camera
    and the boxes, cut out by an alpha texture (uvs repeat it twice)."""
    v = [-0.8, 0.05, 0.3, 0.8, 0.05, 0.3, 0.8, 1.5, 0.3, -0.8, 1.5, 0.3]
    return ("AttributeBegin", "  " + material,
            '  Shape "trianglemesh" "integer indices" [0 1 2 0 2 3] "point P" [%s] "float uv" [0 0 2 0 2 2 0 2] '
            '"texture alpha" "%s"' % (" ".join("%g" % a for a in v), texture),
            "AttributeEnd")


def texture_statements(filename, name="checks", uscale=1.0, vscale=1.0):
    """A pbrt "imagemap" spectrum texture of a linear image file."""
    return ('Texture "%s" "spectrum" "imagemap" "string filename" "%s" "float uscale" [%g] "float vscale" [%g]'
            % (name, filename, uscale, vscale),)


def specular_texture_pbrt(texture_file, seed=23, width=64, height=64, spp=16, maxdepth=8, bump_file=None, **kw):
    """pbrt-v3 text of a Cornell box whose textures are also seen through
    delta bounces: the floor, back and left walls textured with
    `texture_file` (uv scale 1 and 2 x 3), the right wall a mirror with uvs
    and splayed vertex normals, a smooth glass panel with uvs and splayed
    normals in front of the room, a mirror box and a glass box without uvs.
    bump_file: an image bump map on the back wall too; kw: more cornell_pbrt
    arguments (the integrator)."""
    texs = texture_statements(texture_file) + texture_statements(texture_file, "fine", 2.0, 3.0)
    mirror_normals = ' "normal N" [-1 -0.12 -0.1 -1 0.1 -0.12 -1 0.12 0.1 -1 -0.1 0.12]'
    walls = {4: ('Material "mirror" "rgb Kr" [0.9 0.85 0.8]', mirror_normals)}
    wall_textures = {0: "fine", 2: "checks", 3: "fine"}
    if bump_file:
        texs += ('Texture "bumps" "float" "imagemap" "string filename" "%s"' % bump_file,)
        walls[2] = ('Material "matte" "texture Kd" "checks" "texture bumpmap" "bumps"', "")
        del wall_textures[2]
    v = [-0.65, 0.05, 0.6, 0.25, 0.05, 0.6, 0.25, 1.45, 0.6, -0.65, 1.45, 0.6]
    n = [-0.12, -0.1, 1, 0.12, -0.1, 1, 0.12, 0.1, 1, -0.12, 0.1, 1]
    panel = ("AttributeBegin",
             '  Material "glass" "float index" [1.5] "rgb Kr" [1 1 1] "rgb Kt" [1 1 1]',
             '  Shape "trianglemesh" "integer indices" [0 1 2 0 2 3] "point P" [%s] "float uv" [0 0 2 0 2 2 0 2]'
             ' "normal N" [%s]' % (" ".join("%g" % x for x in v), " ".join("%g" % x for x in n)),
             "AttributeEnd")
    return cornell_pbrt(seed=seed, width=width, height=height, spp=spp, maxdepth=maxdepth, box_materials=DELTA_BOXES,
                        textures=texs, wall_textures=wall_textures, wall_materials=walls, extra_shapes=panel, **kw)


def texture_glass_panel(s):
    """Gives the flattened scene of specular_texture_pbrt's glass panel (its
    last object) the back wall's texture as Kr (uv scale 2 x 3) and Kt: the
    pbrt loader reads constant Kr and Kt only."""
    mats = s.materials
    checks = int(mats["reflectance_texture"][s.objects["material_index"][2]])
    g = int(s.objects["material_index"][-1])
    assert checks > 0 and int(mats["type"][g]) == 7 and not float(mats["u_roughness"][g]) > 0  # smooth glass
    mats["reflectance_texture"][g] = checks
    mats["reflectance_uv_scale"][g] = (2.0, 3.0)
    mats["transmittance_texture"][g] = checks
    mats["transmittance_uv_scale"][g] = (1.0, 1.0)
    return s


def environment_statements(mapname, scale=(1, 1, 1), samples=1):
    """pbrt statements of an infinite light with the given map, turned so that
    the map's pole points along +y."""
    return ("AttributeBegin", "  Rotate -90 1 0 0",
            '  LightSource "infinite" "string mapname" "%s" "integer nsamples" [%d] "rgb L" [%g %g %g]'
            % ((mapname, samples) + tuple(scale)),
            "AttributeEnd")


def make_diffuse_transmission(flat, obj=5, reflectance=(0.6, 0.5, 0.4), transmittance=(0.3, 0.4, 0.5),
                              scale=(1.2, 1.0, 0.9)):
    """Turns object `obj`'s material (object 5 is cornell_pbrt's short box)
    into a diffuse-transmission material (a YAR material pbrt has no name for)."""
    m = flat.materials.copy()
    o = flat.objects.copy()
    k = int(o[obj]["material_index"])
    m[k] = np.zeros((), m.dtype)
    m[k]["type"] = 3  # YAR_MATERIAL_DIFFUSE_TRANSMISSION
    m[k]["reflectance"] = reflectance
    m[k]["transmittance"] = transmittance
    m[k]["diffuse"] = scale
    o[obj]["material_type"] = 3
    flat.materials = m
    flat.objects = o
    return flat


UPPER_LIGHT = (0.8, 2.3, 4.0)


def hexagon(center, radius, axis, facing):
    """A 6-triangle fan in the plane normal to `axis` (0 x, 1 y, 2 z), wound
    so that its geometric normal points along `facing` (+1 or -1)."""
    c = np.asarray(center, np.float32)
    u, w = [(1, 2), (2, 0), (0, 1)][axis]
    ring = []
    for k in range(6):
        t = 2 * math.pi * k / 6
        p = c.copy()
        p[u] += radius * math.cos(t)
        p[w] += radius * math.sin(t)
        ring.append(p)
    v = np.array([c] + ring, np.float32)
    idx = [[0, 1 + k, 1 + (k + 1) % 6] for k in range(6)]
    e1, e2 = v[1] - v[0], v[2] - v[0]
    if np.cross(e1, e2)[axis] * facing < 0:
        idx = [[a, b2, b1] for a, b1, b2 in idx]
    return v, np.array(idx, np.int32)


def _mesh_lights():
    ceiling_v, ceiling_i = hexagon((0.45, 1.97, 0.35), 0.12, 1, -1)
    wall_v, wall_i = hexagon((-0.98, 1.2, -0.3), 0.15, 0, +1)
    wall_n = np.tile(np.array([[1.0, 0.0, 0.0]], np.float32), (wall_v.shape[0], 1))
    return ((ceiling_v, ceiling_i, None, (6.0, 5.5, 5.0)), (wall_v, wall_i, wall_n, (1.5, 2.0, 3.0)))


# Two small emitting spheres: one in the open, one close to the tall box.
SPHERE_LIGHTS = (((0.55, 1.35, 0.55), 0.08, (5.0, 4.5, 4.0)), ((-0.2, 0.5, 0.2), 0.05, (2.0, 3.0, 4.0)))

def add_sphere_lights(flat, lights=SPHERE_LIGHTS, level=2, threads=0):
    """Adds emitting spheres to a flat scene: per light an icosphere mesh of
    the light's radius (the reference tessellates pbrt spheres the same way,
    here at a lower level), an object translated to the center that carries
    the sphere light, and the Diffuse_Sphere_Light record; the kd-trees are
    rebuilt with the reference builder."""
    from .scene import Mesh, SPHERE_LIGHT_DTYPE, make_object
    records = np.zeros(len(lights), SPHERE_LIGHT_DTYPE)
    objects = list(flat.objects)
    first = flat.sphere_lights.shape[0]
    for k, (center, radius, radiance) in enumerate(lights):
        v, idx = icosphere(radius, level)
        m = Mesh(v, idx)
        m.bounds, m.nodes = native.build_mesh_kdtree(m.vertices, m.indices, threads)
        flat.meshes.append(m)
        xf = np.array([1, 0, 0, center[0], 0, 1, 0, center[1], 0, 0, 1, center[2]], np.float32)
        objects.append(make_object(len(flat.meshes) - 1, xf, material_type=native.MATERIAL_NULL, material_index=-1,
                                   light_type=native.LIGHT_SPHERE, light_index=first + k))
        records[k]["position"] = center
        records[k]["emitted_radiance"] = radiance
        records[k]["radius"] = radius
        records[k]["sample_count"] = 1
    flat.objects = np.array(objects, flat.objects.dtype)
    flat.sphere_lights = np.concatenate([flat.sphere_lights, records])
    flat.build_scene_kdtree()
    return flat


# A hexagonal light on the ceiling (geometric normal) and one on the left wall
# (vertex normals), both triangle-mesh lights.
MESH_LIGHTS = _mesh_lights()

# A point light low in the room, a spot light from the ceiling onto the boxes
# with a penumbra, and a distant light through the open front.
DELTA_LIGHTS = ('LightSource "point" "point from" [-0.6 0.4 0.6] "rgb I" [0.8 0.6 0.4]',
                'LightSource "spot" "point from" [0.3 1.9 0.2] "point to" [0.2 0 0.1] "float coneangle" [25] '
                '"float conedeltaangle" [8] "rgb I" [3 3 3.5]',
                'LightSource "distant" "point from" [0.4 0.9 2.5] "point to" [0 0 0] "rgb L" [0.6 0.65 0.7]')  # half size, height, radiance


def make_ceiling_refractor(flat, ior=1.0 / 1.5):
    """Turns the ceiling (object 1 of cornell_pbrt's flattened scene) into a
    perfect refractor.  Its normal faces up, so rays from the room leave the
    medium with eta = ior < 1 and never meet total internal reflection (the
    reference asserts there); nothing above the ceiling but the upper light
    sends rays back."""
    m = flat.materials.copy()
    o = flat.objects.copy()
    k = int(o[1]["material_index"])
    m[k]["type"] = 1  # YAR_MATERIAL_PERFECT_REFRACTOR
    m[k]["index_of_refraction"] = np.float32(ior)
    o[1]["material_type"] = 1
    flat.materials = m
    flat.objects = o
    return flat


GGX_BOXES = ('Material "metal" "float roughness" [0.2] "rgb eta" [0.2 0.92 1.1] "rgb k" [3.9 2.45 2.14]',
             'Material "glass" "float uroughness" [0.3] "float vroughness" [0.3] "float index" [1.5] '
             '"rgb Kr" [1 1 1] "rgb Kt" [1 1 1]')


# ---------------------------------------------------------------- large wavefront scene
METALS = (((0.2, 0.92, 1.1), (3.9, 2.45, 2.14)),    # gold-like
          ((0.27, 0.68, 1.32), (3.61, 2.63, 2.29)),  # copper-like
          ((0.16, 0.14, 0.13), (4.0, 3.2, 2.5)))     # silver-like


def _pbrt_quad_uvs():
    # pbrt-v3 default uvs of a 4-vertex mesh (src/lib/pbrt_scene.cpp:305-315)
    return np.array([[0, 0], [1, 0], [1, 1], [1, 0]], np.float32)


def large_scene(seed=1, width=1920, height=1080, spp=64, maxdepth=16, meshes=200, level=5, lights=64, build=True,
                threads=0):
    """The plain-wavefront workload: the Cornell room and boxes plus `meshes`
    icosphere copies (level 5: 20,480 triangles each, ~4.1M in total), half
    Lambertian and half GGX (conductors and rough dielectrics, roughness
    U[0.05, 0.5], IOR U[1.3, 1.7], pbrt-v3 roughness remapping), lit only by
    `lights` 0.1 x 0.1 ceiling quads of radiance log-uniform in [1, 100].
    Rendered at width x height, spp samples, maxdepth bounces, Russian roulette
    from bounce 3 (the reference defaults)."""
    from . import native as N
    from .scene import LIGHT_DTYPE, MATERIAL_DTYPE, CAMERA_DTYPE, default_config
    rng = np.random.default_rng(seed)
    s = FlatScene()
    objects, materials, rect_lights = [], [], []

    def add_material(kind):
        m = np.zeros((), MATERIAL_DTYPE)
        if kind == "matte":
            m["type"] = N.MATERIAL_DIFFUSE
            m["reflectance"] = rng.uniform(0.2, 0.8, 3)
        elif kind == "metal":
            eta, k = METALS[int(rng.integers(0, len(METALS)))]
            r = rng.uniform(0.05, 0.5)
            m["type"] = N.MATERIAL_METAL
            m["eta"], m["k"], m["eta_i"] = eta, k, 1.0
            m["u_roughness"] = m["v_roughness"] = r
        else:
            r = rng.uniform(0.05, 0.5)
            m["type"] = N.MATERIAL_GLASS
            m["reflectance"] = m["transmittance"] = (1.0, 1.0, 1.0)
            m["index_of_refraction"] = rng.uniform(1.3, 1.7)
            m["u_roughness"] = m["v_roughness"] = r
        materials.append(m)
        return int(m["type"]), len(materials) - 1

    walls = [
        _quad((-1, 0, -1), (1, 0, -1), (1, 0, 1), (-1, 0, 1)),
        _quad((-1, 2, -1), (-1, 2, 1), (1, 2, 1), (1, 2, -1)),
        _quad((-1, 0, -1), (-1, 2, -1), (1, 2, -1), (1, 0, -1)),
        _quad((-1, 0, -1), (-1, 0, 1), (-1, 2, 1), (-1, 2, -1)),
        _quad((1, 0, -1), (1, 2, -1), (1, 2, 1), (1, 0, 1)),
    ]
    for v, i in walls:
        s.meshes.append(Mesh(v, i, uvs=_pbrt_quad_uvs()))
        t, k = add_material("matte")
        objects.append(make_object(len(s.meshes) - 1, material_type=t, material_index=k))
    for center, size in (((0.35, 0, 0.3), (0.6, 0.6, 0.6)), ((-0.35, 0, -0.35), (0.6, 1.2, 0.6))):
        v, i = _box(center, size, rng.uniform(0.0, 30.0))
        s.meshes.append(Mesh(v, i))
        t, k = add_material("matte")
        objects.append(make_object(len(s.meshes) - 1, material_type=t, material_index=k))
    sv, si = icosphere(1.0, level)
    for _ in range(meshes):
        r = np.float32(rng.uniform(0.03, 0.12))
        c = rng.uniform((-0.85, 0.1, -0.85), (0.85, 1.8, 0.85)).astype(np.float32)
        s.meshes.append(Mesh(sv * r, si))
        kind = "matte" if rng.random() < 0.5 else ("metal" if rng.random() < 0.5 else "glass")
        t, k = add_material(kind)
        m = np.array([1, 0, 0, c[0], 0, 1, 0, c[1], 0, 0, 1, c[2]], np.float32)
        w = np.array([1, 0, 0, -c[0], 0, 1, 0, -c[1], 0, 0, 1, -c[2]], np.float32)
        objects.append(make_object(len(s.meshes) - 1, m, w, material_type=t, material_index=k))
    side = int(math.ceil(math.sqrt(lights)))
    h = 0.05
    for j in range(lights):
        cx = -0.8 + 1.6 * ((j % side) + 0.5) / side
        cz = -0.8 + 1.6 * ((j // side) + 0.5) / side
        v, i = _quad((cx - h, 1.98, cz - h), (cx + h, 1.98, cz - h), (cx + h, 1.98, cz + h), (cx - h, 1.98, cz + h))
        s.meshes.append(Mesh(v, i, uvs=_pbrt_quad_uvs()))
        L = np.zeros((), LIGHT_DTYPE)
        # rectangle frame: x along +x, y along +z, normal (x cross y) = -y (facing down)
        L["light_to_world"] = (1, 0, 0, cx, 0, 0, -1, 1.98, 0, 1, 0, cz)
        L["emitted_radiance"] = [float(np.exp(rng.uniform(np.log(1.0), np.log(100.0))))] * 3
        L["size"] = (2 * h, 2 * h)
        L["sample_count"] = 1
        rect_lights.append(L)
        objects.append(make_object(len(s.meshes) - 1, material_type=N.MATERIAL_NULL, material_index=-1,
                                   light_type=N.LIGHT_RECT, light_index=len(rect_lights) - 1))
    s.objects = np.array(objects)
    s.materials = np.array(materials, MATERIAL_DTYPE)
    s.rect_lights = np.array(rect_lights, LIGHT_DTYPE)
    cam = np.zeros((), CAMERA_DTYPE)
    cam["camera_to_world"] = (1, 0, 0, 0, 0, 1, 0, 1, 0, 0, 1, 3.5)
    cam["image_extent"] = (width, height)
    vert = np.float32(math.tan(math.radians(20.0)))
    cam["vert_half_dist"] = vert
    cam["horz_half_dist"] = np.float32(np.float32(width) / np.float32(height)) * vert
    cam["z_is_up"] = 0
    s.camera = cam
    k = int(math.ceil(math.sqrt(spp)))
    s.config = default_config(width, height, k, k, maxdepth)
    if build:
        s.build_kdtrees(threads)
    return s


# ---------------------------------------------------------------- hard-lighting room (learned proposal)
def _grid(origin, du, dv, n, hole=None):
    """n x n quads spanning origin + [0,1] du + [0,1] dv (two triangles each);
    `hole` = (i0, i1, j0, j1) cell range left open."""
    o, du, dv = (np.asarray(a, np.float64) for a in (origin, du, dv))
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    v = (o + ii[..., None] / n * du + jj[..., None] / n * dv).reshape(-1, 3).astype(np.float32)
    ci, cj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    ci, cj = ci.ravel(), cj.ravel()
    if hole is not None:
        i0, i1, j0, j1 = hole
        keep = ~((ci >= i0) & (ci < i1) & (cj >= j0) & (cj < j1))
        ci, cj = ci[keep], cj[keep]
    a = ci * (n + 1) + cj
    b, c, d = a + (n + 1), a + (n + 1) + 1, a + 1
    idx = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)]).astype(np.int32)
    return v, idx


def hard_lighting_room(seed=1, width=512, height=512, maxdepth=12, cells=200, light_size=0.1, light_height=0.6,
                       build=True, threads=0):
    """The learned-proposal workload: a closed 2 x 2 x 2 room whose six walls
    are tessellated into `cells` x `cells` quads (200: 479,800 triangles, the
    opening cut out) of
    GGX metal (roughness U[0.1, 0.3] per wall, pbrt-v3 remapping), two
    Lambertian boxes inside, and one light_size x light_size area light of
    radiance 1000 light_height above the ceiling, which reaches the room
    only through a 0.1 x 0.1 opening in the ceiling's centre: the opening
    collimates it into a pool on the floor (about 0.75 wide, all penumbra),
    and the rest of the room, the boxes (placed outside the beam) and
    everything the camera sees, is lit only by what that pool and the glossy
    walls reflect.  512 x 512, maxdepth 12, Russian roulette from bounce 3."""
    from . import native as N
    from .scene import LIGHT_DTYPE, MATERIAL_DTYPE, CAMERA_DTYPE, default_config
    rng = np.random.default_rng(seed)
    s = FlatScene()
    objects, materials = [], []
    h = int(round(0.025 * cells))                    # opening half-width in cells (0.05 of the 2-unit wall)
    mid = cells // 2
    walls = [
        ((-1, 0, -1), (2, 0, 0), (0, 0, 2), None),                          # floor
        ((-1, 2, -1), (2, 0, 0), (0, 0, 2), (mid - h, mid + h, mid - h, mid + h)),  # ceiling with the opening
        ((-1, 0, -1), (2, 0, 0), (0, 2, 0), None),                          # back
        ((-1, 0, 1), (2, 0, 0), (0, 2, 0), None),                           # front (behind the camera)
        ((-1, 0, -1), (0, 0, 2), (0, 2, 0), None),                          # left
        ((1, 0, -1), (0, 0, 2), (0, 2, 0), None),                           # right
    ]
    for origin, du, dv, hole in walls:
        v, i = _grid(origin, du, dv, cells, hole)
        s.meshes.append(Mesh(v, i))
        m = np.zeros((), MATERIAL_DTYPE)
        eta, k = METALS[2] if rng.random() < 0.5 else METALS[int(rng.integers(0, 2))]
        m["type"] = N.MATERIAL_METAL
        m["eta"], m["k"], m["eta_i"] = eta, k, 1.0
        m["u_roughness"] = m["v_roughness"] = rng.uniform(0.1, 0.3)
        materials.append(m)
        objects.append(make_object(len(s.meshes) - 1, material_type=N.MATERIAL_METAL,
                                   material_index=len(materials) - 1))
    for center, size in (((0.62, 0, 0.4), (0.45, 0.5, 0.45)), ((-0.62, 0, -0.55), (0.45, 1.0, 0.45))):
        v, i = _box(center, size, rng.uniform(0.0, 30.0))
        s.meshes.append(Mesh(v, i))
        m = np.zeros((), MATERIAL_DTYPE)
        m["type"] = N.MATERIAL_DIFFUSE
        m["reflectance"] = rng.uniform(0.4, 0.8, 3)
        materials.append(m)
        objects.append(make_object(len(s.meshes) - 1, material_type=N.MATERIAL_DIFFUSE,
                                   material_index=len(materials) - 1))
    lh, ly = 0.5 * light_size, 2.0 + light_height
    v, i = _quad((-lh, ly, -lh), (lh, ly, -lh), (lh, ly, lh), (-lh, ly, lh))
    s.meshes.append(Mesh(v, i, uvs=_pbrt_quad_uvs()))
    L = np.zeros((), LIGHT_DTYPE)
    L["light_to_world"] = (1, 0, 0, 0, 0, 0, -1, ly, 0, 1, 0, 0)   # normal -y: facing the opening
    L["emitted_radiance"] = (1000.0, 1000.0, 1000.0)
    L["size"] = (2 * lh, 2 * lh)
    L["sample_count"] = 1
    objects.append(make_object(len(s.meshes) - 1, material_type=N.MATERIAL_NULL, material_index=-1,
                               light_type=N.LIGHT_RECT, light_index=0))
    s.objects = np.array(objects)
    s.materials = np.array(materials, MATERIAL_DTYPE)
    s.rect_lights = np.array([L], LIGHT_DTYPE)
    cam = np.zeros((), CAMERA_DTYPE)
    cam["camera_to_world"] = (1, 0, 0, 0, 0, 1, 0, 1.0, 0, 0, 1, 0.95)
    cam["image_extent"] = (width, height)
    vert = np.float32(math.tan(math.radians(35.0)))
    cam["vert_half_dist"] = vert
    cam["horz_half_dist"] = np.float32(np.float32(width) / np.float32(height)) * vert
    cam["z_is_up"] = 0
    s.camera = cam
    s.config = default_config(width, height, 1, 1, maxdepth)
    if build:
        s.build_kdtrees(threads)
    return s


# ---------------------------------------------------------------- batched scenes
def batch_scenes(seed=4, count=64, maxdepth=8, build=True, threads=0):
    """The batched-render workload: `count` independent scenes built like the
    large wavefront scene (Cornell room and boxes, icosphere copies, half
    Lambertian and half GGX, quad ceiling lights) with triangle counts
    log-uniform in [1K, 200K] (icosphere level 3, 4 or 5 by size),
    resolutions uniform in {128^2, 256^2, 512^2, 1024^2}, samples per pixel
    log-uniform in [4, 256] rounded to a perfect square (the stratified
    sampler's k x k grid), 4-16 lights, maxdepth `maxdepth`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        tris = float(np.exp(rng.uniform(np.log(1e3), np.log(2e5))))
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = float(np.exp(rng.uniform(np.log(4.0), np.log(256.0))))
        k = max(2, min(16, int(round(math.sqrt(spp)))))
        level = 3 if tris < 20000 else (4 if tris < 80000 else 5)
        meshes = max(1, int(round((tris - 36) / (20 * 4 ** level))))
        lights = int(rng.integers(4, 17))
        out.append(large_scene(seed=seed * 1000 + i, width=res, height=res, spp=k * k, maxdepth=maxdepth,
                               meshes=meshes, level=level, lights=lights, build=build, threads=threads))
    return out
