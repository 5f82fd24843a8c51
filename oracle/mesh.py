"""CPU restatement of the reference's sphere boundary sampler -- TEST INFRASTRUCTURE (the
checker of sph_scene_icosphere / sph_scene_sphere in fluids_gb300/csrc/sph_scene.cpp).

  icosphere        mesh/icospheremesh.cpp:10-124 (float arithmetic of Bullet's scalar vector
                   code: midpoints (a + b) * 0.5, normalisation by the reciprocal length)
  sphere_sampling  scene/sphere.cpp:135-171: per triangle 2 * ceil(area / (pi s^2)) points
                   (1 - r1) a + r1 (1 - r2) b + r1 r2 c, r1 = sqrt(u1), r2 = u2, from a
                   default-seeded std::default_random_engine (minstd_rand0) made anew for
                   every triangle, through std::uniform_real_distribution<float>(0, 1)
                   (libstdc++: float(g - 1) / float(2^31 - 2), below 1); then every vertex.
                   Corner reads (offset index, not 3 * index) and the area's third term
                   (ab.x * ac.y - ab.x * ac.y) as written there.

The icosphere is pinned against the reference's own icospheremesh.cpp compiled for the CPU
(oracle/_ref); the sampler is this restatement, bit for bit in float32/float64 as the C++.
"""
import math

import numpy as np

F = np.float32

_FACES = [0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6, 7, 1, 8,
          3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8, 6, 7, 9, 8, 1]


def icosphere(radius, level):
    t = F((1.0 + math.sqrt(5.0)) * 0.5)
    one, zero = F(1), F(0)
    v = [np.array(p, F) for p in ([-one, t, zero], [one, t, zero], [-one, -t, zero], [one, -t, zero],
                                  [zero, -one, t], [zero, one, t], [zero, -one, -t], [zero, one, -t],
                                  [t, zero, -one], [t, zero, one], [-t, zero, -one], [-t, zero, one])]
    f = list(_FACES)
    for _ in range(level):
        nv = list(v)
        nf = []
        for k in range(0, len(f), 3):
            a, b, c = f[k], f[k + 1], f[k + 2]
            ab, bc, ca = len(nv), len(nv) + 1, len(nv) + 2
            nv += [(v[a] + v[b]) * F(0.5), (v[b] + v[c]) * F(0.5), (v[c] + v[a]) * F(0.5)]
            nf += [a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca]
        v, f = nv, nf
    out = []
    for p in v:
        ln = np.sqrt((p[0] * p[0] + p[1] * p[1]) + p[2] * p[2])
        inv = F(1.0) / ln
        out.append((p * inv) * F(radius))
    return np.array(out, F), np.array(f, np.uint32) & 0xFFFF


class _MinStd0:
    def __init__(self):
        self.x = 1

    def uniform(self):
        self.x = (self.x * 16807) % 2147483647
        r = F(self.x - 1) / F(2147483646)   # both sides rounded to float, as libstdc++ does
        return r if r < F(1) else np.nextafter(F(1), F(0))


def sphere_sampling(radius, spacing):
    v, ix = icosphere(radius, 3)
    flat = v.reshape(-1)
    area_particle = F(math.pi * float(np.float64(F(spacing)) ** 2))
    pts = []
    for k in range(0, len(ix) - 2, 3):
        a, b, c = (flat[int(i):int(i) + 3] for i in ix[k:k + 3])
        ab, ac = a - b, a - c
        t0 = np.float64(ab[1] * ac[2] - ab[2] * ac[1]) ** 2
        t1 = np.float64(ab[2] * ac[0] - ab[0] * ac[2]) ** 2
        t2 = np.float64(ab[0] * ac[1] - ab[0] * ac[1]) ** 2
        area = F(0.5 * math.sqrt((t0 + t1) + t2))
        n = int(F(2) * np.ceil(area / area_particle))
        g = _MinStd0()
        for _ in range(n):
            r1 = np.sqrt(g.uniform())
            r2 = g.uniform()
            pts.append(((F(1) - r1) * a + (r1 * (F(1) - r2)) * b) + (r2 * r1) * c)
    pts += list(v)
    out = np.ones((len(pts), 4), F)
    out[:, :3] = np.array(pts, F)
    return out
