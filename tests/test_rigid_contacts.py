"""The host World's rigid contact pipeline (csrc/host/rigid_contacts.cpp:
shape boxes, broad phase, narrow phase, islands and sleep, the contact
solver) against the reference's own World built from its sources
(oracle/_ref), bit for bit: single shape pairs over random poses, the broad
phase over random boxes, and whole scenes stepped for hundreds of steps
(resting, stacking, tumbling, bouncing, piles, compound bodies, sleep).
CPU only; skipped where the reference tree is absent."""
import numpy as np
import pytest

nv = pytest.importorskip("novaphy_gb300._core")

from oracle import oracle  # noqa: E402

BOX, SPHERE, PLANE = 0, 1, 2
IDENT = (1.0, 0.0, 0.0, 0.0)


@pytest.fixture(scope="module")
def ref():
    try:
        return oracle.Ref()
    except FileNotFoundError as e:
        pytest.skip(str(e))


def f32(x):
    return np.asarray(x, np.float32)


def shape(kind, body, half=(0.5, 0.5, 0.5), radius=0.5, normal=(0, 1, 0), offset=0.0,
          lpos=(0, 0, 0), lquat=IDENT, friction=0.5, restitution=0.3):
    return f32([kind, body, *half, radius, *normal, offset, *lpos, *lquat, friction, restitution])


def body(mass, inertia_diag, pos, quat=IDENT):
    i = np.diag(f32(inertia_diag)).reshape(-1)
    return f32([mass, *i, *pos, *quat])


def box_inertia(m, he):
    m, (x, y, z) = np.float32(m), f32(he)
    w, h, d = np.float32(2) * x, np.float32(2) * y, np.float32(2) * z
    c = m / np.float32(12)
    return c * (h * h + d * d), c * (w * w + d * d), c * (w * w + h * h)


def sphere_inertia(m, r):
    i = np.float32(2.0 / 5.0) * np.float32(m) * np.float32(r) * np.float32(r)
    return i, i, i


def transform(pose):
    p = [float(v) for v in pose]
    return nv.Transform(p[:3], [p[4], p[5], p[6], p[3]])


def our_shape(s):
    cs = nv.CollisionShape()
    cs.type = [nv.ShapeType.Box, nv.ShapeType.Sphere, nv.ShapeType.Plane][int(s[0])]
    cs.body_index = int(s[1])
    cs.box_half_extents = s[2:5]
    cs.sphere_radius = float(s[5])
    cs.plane_normal = s[6:9]
    cs.plane_offset = float(s[9])
    cs.local_transform = transform(s[10:17])
    cs.friction = float(s[17])
    cs.restitution = float(s[18])
    return cs


def our_contacts(cs):
    rows = [[*c.position, *c.normal, c.penetration, c.body_a, c.body_b, c.friction,
             c.restitution] for c in cs]
    return f32(rows).reshape(-1, 11)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def random_quat(rng):
    q = rng.normal(size=4).astype(np.float32)
    return q / np.float32(np.linalg.norm(q))


# ---- narrow phase ----

def random_shape(rng, kind, body_index):
    if kind == BOX:
        return shape(BOX, body_index, half=rng.uniform(0.1, 0.8, 3), friction=rng.uniform(0, 1),
                     restitution=rng.uniform(0, 1))
    if kind == SPHERE:
        lpos = rng.uniform(-0.2, 0.2, 3) if rng.random() < 0.3 else (0, 0, 0)
        return shape(SPHERE, body_index, radius=rng.uniform(0.1, 0.8), lpos=lpos,
                     friction=rng.uniform(0, 1), restitution=rng.uniform(0, 1))
    n = rng.normal(size=3).astype(np.float32)
    n = n / np.float32(np.linalg.norm(n))
    return shape(PLANE, -1, normal=n, offset=rng.uniform(-0.3, 0.3), friction=rng.uniform(0, 1),
                 restitution=0.0)


@pytest.mark.parametrize("kinds", [(SPHERE, SPHERE), (SPHERE, PLANE), (PLANE, SPHERE),
                                   (BOX, SPHERE), (SPHERE, BOX), (BOX, PLANE), (PLANE, BOX),
                                   (BOX, BOX), (PLANE, PLANE)])
def test_shape_pairs_match_reference(ref, kinds):
    rng = np.random.default_rng(100 + 10 * kinds[0] + kinds[1])
    hits = 0
    for trial in range(400):
        sa, sb = random_shape(rng, kinds[0], 0), random_shape(rng, kinds[1], 1)
        pa = f32([*rng.uniform(-0.5, 0.5, 3), *random_quat(rng)])
        pb = f32([*rng.uniform(-0.5, 0.5, 3) * (0.3 if trial % 4 == 0 else 1.5),
                  *random_quat(rng)])
        if trial % 7 == 0:  # axis-aligned poses: faces parallel, ties between axes
            pa[3:] = IDENT
            pb[3:] = IDENT
        hit_r, c_r = ref.collide(sa, pa, sb, pb)
        hit_o, c_o = nv.collide_shapes(our_shape(sa), transform(pa), our_shape(sb), transform(pb))
        c_o = our_contacts(c_o)
        assert hit_o == hit_r, trial
        assert c_o.shape == c_r.shape, trial
        np.testing.assert_array_equal(bits(c_o), bits(c_r), err_msg=f"trial {trial}")
        hits += hit_r
    if kinds != (PLANE, PLANE):
        assert hits > 40  # the poses exercise contacts, not only misses


def test_sphere_inside_box_takes_the_nearest_face(ref):
    sa = shape(BOX, 0, half=(0.5, 0.3, 0.7))
    sb = shape(SPHERE, 1, radius=0.2)
    for centre in [(0.1, 0.05, 0.0), (0.0, -0.2, 0.1), (0.3, 0.0, 0.65), (0.0, 0.0, 0.0)]:
        pa = f32([0, 0, 0, *IDENT])
        pb = f32([*centre, *IDENT])
        hit_r, c_r = ref.collide(sa, pa, sb, pb)
        _, c_o = nv.collide_shapes(our_shape(sa), transform(pa), our_shape(sb), transform(pb))
        assert hit_r
        np.testing.assert_array_equal(bits(our_contacts(c_o)), bits(c_r))


# ---- broad phase ----

@pytest.mark.parametrize("seed", range(6))
def test_broad_phase_pairs_match_reference(ref, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 60))
    lo = np.round(rng.uniform(-3, 3, (n, 3)) * 4) / 4  # quantised: shared end points
    hi = lo + np.round(rng.uniform(0, 1.5, (n, 3)) * 4) / 4
    boxes = f32(np.concatenate([lo, hi], 1))
    fixed = (rng.random(n) < 0.3).astype(np.int32)
    want = ref.sap(boxes, fixed)
    sap = nv.SweepAndPrune()
    sap.update([nv.AABB(b[:3], b[3:]) for b in boxes], [bool(x) for x in fixed])
    got = np.array([[p.body_a, p.body_b] for p in sap.get_pairs()], np.int32).reshape(-1, 2)
    np.testing.assert_array_equal(got, want)


# ---- whole worlds ----

DEFAULT = (30, 0.3, 0.005, 1, 0, 0.01, 0.5, 0.8)
GRAVITY = (0.0, -9.81, 0.0)


def run_ours(bodies, shapes, lin, ang, settings, gravity, dt, nsteps):
    mb = nv.ModelBuilder()
    for b in bodies:
        rb = nv.RigidBody()
        rb.mass = float(b[0])
        rb.inertia = b[1:10].reshape(3, 3)
        mb.add_body(rb, transform(b[10:17]))
    for s in shapes:
        mb.add_shape(our_shape(s))
    st = nv.SolverSettings()
    (st.velocity_iterations, st.baumgarte, st.slop, warm, sleep, st.sleep_energy_threshold,
     st.sleep_time_required, st.sleep_ema_alpha) = settings
    st.warm_starting, st.sleep_enabled = bool(warm), bool(sleep)
    w = nv.World(mb.build(), st)
    w.set_gravity(list(gravity))
    for k in range(len(bodies)):
        w.state.set_linear_velocity(k, lin[k])
        w.state.set_angular_velocity(k, ang[k])
    counts = []
    for _ in range(nsteps):
        w.step(dt)
        counts.append(len(w.contacts))
    tr = w.state.transforms
    pos = f32([t.position for t in tr])
    quat = f32([[t.rotation[3], *t.rotation[:3]] for t in tr])
    return (pos, quat, f32(w.state.linear_velocities), f32(w.state.angular_velocities),
            np.array(counts, np.int32), np.array(w.state.sleeping, np.int32))


def check_world(ref, bodies, shapes, lin=None, ang=None, settings=DEFAULT, gravity=GRAVITY,
                dt=1.0 / 120.0, nsteps=240):
    bodies, shapes = f32(bodies), f32(shapes)
    lin = f32(np.zeros((len(bodies), 3)) if lin is None else lin)
    ang = f32(np.zeros((len(bodies), 3)) if ang is None else ang)
    want = ref.rigid_world(bodies, shapes, lin, ang, settings, gravity, dt, nsteps)
    got = run_ours(bodies, shapes, lin, ang, settings, gravity, dt, nsteps)
    names = ["position", "rotation", "linear velocity", "angular velocity", "contacts/step",
             "sleeping"]
    for name, g, r in zip(names, got, want):
        if g.dtype == np.float32:
            np.testing.assert_array_equal(bits(g), bits(r), err_msg=name)
        else:
            np.testing.assert_array_equal(g, r, err_msg=name)
    return got


GROUND = shape(PLANE, -1, friction=0.5, restitution=0.0)


def test_box_rests_on_ground(ref):
    he = (0.5, 0.5, 0.5)
    got = check_world(ref, [body(1.0, box_inertia(1.0, he), (0, 5, 0))], [GROUND, shape(BOX, 0)])
    assert 0.3 < got[0][0, 1] < 1.0
    assert got[4][-1] == 4  # four corners on the ground


def test_sphere_rests_on_ground(ref):
    got = check_world(ref, [body(1.0, sphere_inertia(1.0, 0.5), (0, 3, 0))],
                      [GROUND, shape(SPHERE, 0)], nsteps=360)
    assert 0.3 < got[0][0, 1] < 1.0


def test_two_boxes_stack(ref):
    he = (0.5, 0.5, 0.5)
    bodies = [body(1.0, box_inertia(1.0, he), (0, 1.0 + 1.5 * i, 0)) for i in range(2)]
    shapes = [GROUND, shape(BOX, 0), shape(BOX, 1)]
    got = check_world(ref, bodies, shapes, settings=(15, *DEFAULT[1:]), nsteps=360)
    assert got[0][1, 1] > got[0][0, 1]


def test_tumbling_box_lands_on_edges_and_corners(ref):
    he = (0.6, 0.25, 0.4)
    q = f32([0.9, 0.3, 0.2, 0.25])
    q = q / np.float32(np.linalg.norm(q))
    check_world(ref, [body(2.0, box_inertia(2.0, he), (0.1, 1.5, -0.2), q)],
                [GROUND, shape(BOX, 0, half=he, friction=0.7)], lin=[(1.0, 0.0, 0.5)],
                ang=[(2.0, -1.0, 3.0)], nsteps=300)


def test_bouncing_sphere_uses_restitution(ref):
    got = check_world(ref, [body(1.0, sphere_inertia(1.0, 0.3), (0, 2.5, 0))],
                      [shape(PLANE, -1, restitution=0.8), shape(SPHERE, 0, radius=0.3,
                                                               restitution=0.9)],
                      lin=[(0.5, 0.0, 0.0)], nsteps=240)
    assert got[0][0, 1] > 0.25


def test_pile_of_spheres_and_boxes_with_a_static_body(ref):
    rng = np.random.default_rng(7)
    bodies, shapes = [], [GROUND]
    # a static box (mass 0) the pile falls onto, then spheres and boxes
    bodies.append(body(0.0, (0, 0, 0), (0.0, 0.4, 0.0)))
    shapes.append(shape(BOX, 0, half=(0.6, 0.4, 0.6)))
    for k in range(1, 9):
        pos = (rng.uniform(-0.6, 0.6), 1.2 + 0.6 * k, rng.uniform(-0.6, 0.6))
        q = random_quat(rng)
        if k % 2:
            r = float(rng.uniform(0.15, 0.35))
            bodies.append(body(1.0, sphere_inertia(1.0, r), pos, q))
            shapes.append(shape(SPHERE, k, radius=r, friction=0.4, restitution=0.2))
        else:
            he = tuple(rng.uniform(0.15, 0.35, 3))
            bodies.append(body(1.5, box_inertia(1.5, he), pos, q))
            shapes.append(shape(BOX, k, half=he, friction=0.6, restitution=0.1))
    got = check_world(ref, bodies, shapes, nsteps=400)
    assert got[4].max() >= 8


def test_compound_body_and_no_warm_start(ref):
    # one body carrying a box and an offset sphere, dropped on the ground
    he = (0.4, 0.2, 0.3)
    lq = f32([0.96, 0.0, 0.28, 0.0])
    lq = lq / np.float32(np.linalg.norm(lq))
    shapes = [GROUND, shape(BOX, 0, half=he, lquat=lq), shape(SPHERE, 0, radius=0.25,
                                                            lpos=(0.5, 0.1, 0.0))]
    settings = (12, 0.2, 0.01, 0, 0, 0.01, 0.5, 0.8)
    check_world(ref, [body(3.0, box_inertia(3.0, he), (0, 1.0, 0))], shapes, ang=[(0, 0, 1.5)],
                settings=settings, nsteps=300)


def test_falling_stack_sleeps_and_wakes(ref):
    # the boxes land on one another, the bottom one falls asleep, the upper
    # ones topple off (waking islands on the way); the sphere sleeps alone
    he = (0.5, 0.5, 0.5)
    bodies = [body(1.0, box_inertia(1.0, he), (0.05 * i, 0.8 + 1.3 * i, 0)) for i in range(3)]
    bodies.append(body(1.0, sphere_inertia(1.0, 0.3), (4.0, 1.0, 0.0)))
    shapes = [GROUND] + [shape(BOX, i) for i in range(3)] + [shape(SPHERE, 3, radius=0.3)]
    settings = (20, 0.3, 0.005, 1, 1, 0.05, 0.3, 0.8)
    got = check_world(ref, bodies, shapes, settings=settings, nsteps=480)
    assert got[5].sum() >= 1  # the sleep path ran: some body is asleep at the end


def test_world_defaults_match_reference_settings():
    s = nv.SolverSettings()
    assert (s.velocity_iterations, s.warm_starting, s.sleep_enabled) == (30, True, False)
    assert abs(s.baumgarte - 0.3) < 1e-7 and abs(s.slop - 0.005) < 1e-9
    assert abs(s.sleep_energy_threshold - 0.01) < 1e-9
    assert abs(s.sleep_time_required - 0.5) < 1e-9 and abs(s.sleep_ema_alpha - 0.8) < 1e-7


def test_scattered_pile_sleeps_island_by_island(ref):
    # ten bodies dropped over a 4 m square: several islands, some asleep at
    # the end while others still move
    rng = np.random.default_rng(11)
    bodies, shapes = [], [GROUND]
    for k in range(10):
        pos = (rng.uniform(-2, 2), 0.3 + 0.8 * k, rng.uniform(-2, 2))
        if k % 2:
            r = float(rng.uniform(0.15, 0.35))
            bodies.append(body(1.0, sphere_inertia(1.0, r), pos, random_quat(rng)))
            shapes.append(shape(SPHERE, k, radius=r, friction=0.8))
        else:
            he = tuple(rng.uniform(0.15, 0.35, 3))
            bodies.append(body(1.5, box_inertia(1.5, he), pos, random_quat(rng)))
            shapes.append(shape(BOX, k, half=he, friction=0.8, restitution=0.1))
    got = check_world(ref, bodies, shapes, settings=(20, 0.3, 0.005, 1, 1, 0.05, 0.3, 0.8),
                      nsteps=600)
    assert 1 <= got[5].sum() < len(bodies)


def test_thousand_box_stacks(ref):
    # 10 x 10 columns of 10 boxes settling (about 2,000 contacts a step):
    # the broad phase, the contact order and the solver sweep at scale
    rng = np.random.default_rng(3)
    bodies, shapes = [], [GROUND]
    he = (0.2, 0.2, 0.2)
    for i in range(10):
        for j in range(10):
            for k in range(10):
                bodies.append(body(1.0, box_inertia(1.0, he),
                                   (i * 0.5 + rng.uniform(0, 0.05), 0.25 + k * 0.41, j * 0.5)))
                shapes.append(shape(BOX, len(bodies) - 1, half=he))
    got = check_world(ref, bodies, shapes, settings=(10, *DEFAULT[1:]), nsteps=60)
    assert got[4][-1] > 1500
