"""Generates the golden fixtures under tests/golden/ by running the reference.

The reference is built from its own sources by oracle/ref_build/Makefile into
oracle/_ref/<variant>/libode.a; this script compiles tests/golden/gen_golden.cpp
against it, writes seeded inputs, runs it and packs the outputs as .npz.

    python tests/golden/make_golden.py --ref <reference source tree>

Only this container has the reference sources; the fixtures it writes are
committed so that tests elsewhere need neither the reference nor this script.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ode_gb300 import scenes  # noqa: E402

REF_OUT = os.path.join(ROOT, "oracle", "_ref")
SHIM = os.path.join(ROOT, "oracle", "ref_build", "shim")


def build(ref: str) -> dict:
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref_build"),
                           f"REF={ref}", "-j8"])
    exes = {}
    for variant, prec in (("single", "dIDESINGLE"), ("single_noreorder", "dIDESINGLE"),
                          ("double", "dIDEDOUBLE")):
        exe = os.path.join(REF_OUT, variant, "gen_golden")
        subprocess.check_call(["g++", "-O2", "-ffp-contract=off", f"-D{prec}", f"-I{SHIM}",
                               f"-I{ref}/include", os.path.join(HERE, "gen_golden.cpp"),
                               os.path.join(REF_OUT, variant, "libode.a"), "-lpthread", "-o", exe])
        exes[variant] = exe
    return exes


def run(exe: str, mode: str, arrays: list, messages: list | None = None) -> bytes:
    """Runs gen_golden MODE on the arrays; the reference's messages (stderr)
    are appended to `messages` when given."""
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            for a in arrays:
                f.write(np.ascontiguousarray(a).tobytes())
        p = subprocess.run([exe, mode, fin, fout], stderr=subprocess.PIPE, text=True, check=True)
        if messages is not None:
            messages.append(p.stderr)
        with open(fout, "rb") as f:
            return f.read()


class Reader:
    def __init__(self, buf: bytes):
        self.buf, self.off = buf, 0

    def take(self, dtype, count):
        a = np.frombuffer(self.buf, dtype=dtype, count=count, offset=self.off)
        self.off += a.nbytes
        return a.copy()

    def done(self):
        return self.off >= len(self.buf)


# --------------------------------------------------------------------- colliders
EXTENT = {scenes.SPHERE: lambda d: d[0], scenes.BOX: lambda d: 0.5 * np.linalg.norm(d[:3]),
          scenes.CAPSULE: lambda d: d[0] + 0.5 * d[1]}


def rand_dims(rng, cls):
    d = np.zeros(4, np.float32)
    if cls == scenes.SPHERE:
        d[0] = rng.uniform(0.05, 0.6)
    elif cls == scenes.BOX:
        d[:3] = rng.uniform(0.1, 1.2, size=3)
    elif cls == scenes.CAPSULE:
        d[0] = rng.uniform(0.05, 0.4)
        d[1] = rng.uniform(0.0, 1.0)
    return d


def rand_R(rng, kind):
    if kind == 0:
        q = scenes.random_quats(rng, 1)[0]
    elif kind == 1:  # yaw only (stack-like)
        a = rng.uniform(-0.2, 0.2)
        q = np.array([np.cos(a / 2), 0, 0, np.sin(a / 2)], np.float32)
    else:            # axis aligned
        q = np.array([1, 0, 0, 0], np.float32)
    return scenes.quat_to_R(q)


def collider_corpus(seed=7, per_combo=300):
    rng = np.random.default_rng(seed)
    solids = [scenes.SPHERE, scenes.BOX, scenes.CAPSULE]
    combos = [(a, b) for a in solids for b in solids] + \
             [(a, scenes.PLANE) for a in solids] + [(scenes.PLANE, a) for a in solids]
    cls, flags, pos, R, dims = [], [], [], [], []
    for (c1, c2) in combos:
        for k in range(per_combo):
            rk = k % 3
            maxc = int(rng.choice([1, 2, 3, 4, 4, 4, 5, 8]))
            if scenes.PLANE in (c1, c2):
                solid = c2 if c1 == scenes.PLANE else c1
                ds = rand_dims(rng, solid)
                Rs = rand_R(rng, rk)
                ps = rng.uniform(-2, 2, size=3).astype(np.float32)
                if rk == 0:
                    n = rng.normal(size=3)
                    n /= np.linalg.norm(n)
                else:
                    n = np.zeros(3)
                    n[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
                ext = EXTENT[solid](ds)
                dd = float(n @ ps) + rng.uniform(-ext, 1.3 * ext)
                dp = np.array([n[0], n[1], n[2], dd], np.float32)
                zero3, I12 = np.zeros(3, np.float32), scenes.quat_to_R(np.array([1, 0, 0, 0], np.float32))
                if c1 == scenes.PLANE:
                    pos.append([zero3, ps]); R.append([I12, Rs]); dims.append([dp, ds])
                else:
                    pos.append([ps, zero3]); R.append([Rs, I12]); dims.append([ds, dp])
            else:
                d1, d2 = rand_dims(rng, c1), rand_dims(rng, c2)
                R1, R2 = rand_R(rng, rk), rand_R(rng, rk)
                p1 = rng.uniform(-1, 1, size=3).astype(np.float32)
                if rk == 0:
                    u = rng.normal(size=3)
                    u /= np.linalg.norm(u)
                    dist = (EXTENT[c1](d1) + EXTENT[c2](d2)) * rng.uniform(0.05, 1.05)
                    p2 = (p1 + u * dist).astype(np.float32)
                else:
                    # resting-contact geometry: geom 2 above geom 1 along z
                    h1 = d1[2] / 2 if c1 == scenes.BOX else (d1[0] if c1 == scenes.SPHERE else d1[0] + d1[1] / 2)
                    h2 = d2[2] / 2 if c2 == scenes.BOX else (d2[0] if c2 == scenes.SPHERE else d2[0] + d2[1] / 2)
                    off = rng.uniform(-0.3, 0.3, size=2) * min(EXTENT[c1](d1), EXTENT[c2](d2))
                    p2 = (p1 + np.array([off[0], off[1], h1 + h2 - rng.uniform(-0.01, 0.05)])).astype(np.float32)
                pos.append([p1, p2]); R.append([R1, R2]); dims.append([d1, d2])
            cls.append([c1, c2]); flags.append(maxc)
    # hand-made edge cases
    I12 = scenes.quat_to_R(np.array([1, 0, 0, 0], np.float32))
    edge = []
    edge.append(((0, 0), 4, [[0, 0, 0], [0, 0, 0]], [[.5, 0, 0, 0], [.3, 0, 0, 0]]))      # coincident spheres
    edge.append(((0, 1), 4, [[0.1, 0, 0.05], [0, 0, 0]], [[.2, 0, 0, 0], [1, 1, 1, 0]]))  # sphere centre in box
    edge.append(((1, 0), 4, [[0, 0, 0], [0.1, 0, 0.05]], [[1, 1, 1, 0], [.2, 0, 0, 0]]))
    edge.append(((1, 1), 8, [[0, 0, 0], [0, 0, 0.99]], [[1, 1, 1, 0], [1, 1, 1, 0]]))     # aligned stack, 8 slots
    edge.append(((1, 1), 4, [[0, 0, 0], [0, 0, 1.0]], [[1, 1, 1, 0], [1, 1, 1, 0]]))      # exactly touching
    edge.append(((1, 1), 1, [[0, 0, 0], [0.02, 0.01, 0.98]], [[1, 1, 1, 0], [1, 1, 1, 0]]))
    edge.append(((2, 2), 4, [[0, 0, 0], [0.1, 0, 0]], [[.2, 1, 0, 0], [.2, 1, 0, 0]]))    # parallel capsules
    edge.append(((2, 2), 1, [[0, 0, 0], [0.1, 0, 0]], [[.2, 1, 0, 0], [.2, 1, 0, 0]]))
    edge.append(((2, 1), 4, [[0, 0, 0], [0, 0, 0]], [[.2, 1, 0, 0], [1, 1, 2, 0]]))       # capsule axis inside box
    edge.append(((1, 2), 4, [[0, 0, 0], [0, 0, 0]], [[1, 1, 2, 0], [.2, 1, 0, 0]]))
    edge.append(((2, 0), 4, [[0, 0, 0], [0, 0, 0.4]], [[.2, 1, 0, 0], [.3, 0, 0, 0]]))
    for (cc, mc, pp, dd) in edge:
        cls.append(list(cc)); flags.append(mc)
        pos.append([np.array(pp[0], np.float32), np.array(pp[1], np.float32)])
        R.append([I12, I12]); dims.append([np.array(dd[0], np.float32), np.array(dd[1], np.float32)])
    cls = np.array(cls, np.int32)
    flags = np.array(flags, np.int32)
    pos = np.array(pos, np.float32).reshape(-1, 2, 3)
    R = np.array(R, np.float32).reshape(-1, 2, 12)
    dims = np.array(dims, np.float32).reshape(-1, 2, 4)
    return cls, flags, pos, R, dims


def gen_colliders(exes):
    cls, flags, pos, R, dims = collider_corpus()
    n = cls.shape[0]
    out = Reader(run(exes["single"], "colliders",
                     [np.array([n], np.int32), cls, flags, pos, R, dims]))
    count = out.take(np.int32, n)
    code = out.take(np.int32, n)
    cpos = out.take(np.float32, 24 * n).reshape(n, 8, 3)
    cnrm = out.take(np.float32, 24 * n).reshape(n, 8, 3)
    cdep = out.take(np.float32, 8 * n).reshape(n, 8)
    swap = out.take(np.int32, 8 * n).reshape(n, 8)
    side = out.take(np.int32, 16 * n).reshape(n, 8, 2)
    assert out.done()
    np.savez_compressed(os.path.join(HERE, "colliders.npz"), cls=cls, flags=flags, pos=pos, R=R,
                        dims=dims, count=count, code=code, cpos=cpos, cnrm=cnrm, cdep=cdep,
                        swap=swap, side=side)
    print(f"colliders: {n} cases, {int(count.sum())} contacts, "
          f"{int((count > 0).sum())} touching")


# --------------------------------------------------------------------- space
def space_case(rng, n, spread):
    cls = rng.choice([scenes.SPHERE, scenes.BOX, scenes.CAPSULE], size=n).astype(np.int32)
    pos = rng.uniform(-spread, spread, size=(n, 3)).astype(np.float32)
    R = scenes.quat_to_R(scenes.random_quats(rng, n))
    dims = np.zeros((n, 4), np.float32)
    scale = np.exp(rng.uniform(np.log(0.02), np.log(3.0), size=n)).astype(np.float32)
    for i in range(n):
        dims[i] = rand_dims(rng, cls[i]) * scale[i]
    # a few planes (infinite AABBs go to the reference's big-box list)
    npl = 3
    pl = np.array([[0, 0, 1, -spread * 0.5], [1, 0, 0, -spread * 0.7], [0.6, 0.8, 0, 0]], np.float32)
    cls = np.concatenate([cls, np.full(npl, scenes.PLANE, np.int32)])
    pos = np.concatenate([pos, np.zeros((npl, 3), np.float32)])
    R = np.concatenate([R, np.tile(scenes.quat_to_R(np.array([1, 0, 0, 0], np.float32)), (npl, 1))])
    dims = np.concatenate([dims, pl])
    return cls, pos, R, dims


def gen_space(exes):
    rng = np.random.default_rng(11)
    out = {}
    for ci, (n, spread, lv) in enumerate([(300, 4.0, (-3, 10)), (2000, 12.0, (-3, 10)),
                                          (1000, 6.0, (-1, 3)), (500, 3.0, (0, 0))]):
        cls, pos, R, dims = space_case(rng, n, spread)
        ng = cls.shape[0]
        r = Reader(run(exes["single"], "space", [np.array([ng, lv[0], lv[1]], np.int32), cls, pos, R, dims]))
        npairs = int(r.take(np.int32, 1)[0])
        pairs = r.take(np.int32, 2 * npairs).reshape(-1, 2)
        assert r.done()
        out[f"c{ci}_cls"], out[f"c{ci}_pos"], out[f"c{ci}_R"], out[f"c{ci}_dims"] = cls, pos, R, dims
        out[f"c{ci}_levels"] = np.array(lv, np.int32)
        out[f"c{ci}_pairs"] = pairs
        print(f"space case {ci}: {ng} geoms, {npairs} callback pairs, "
              f"{len(set(map(tuple, pairs.tolist())))} distinct")
    out["ncases"] = np.array([4], np.int32)
    np.savez_compressed(os.path.join(HERE, "space.npz"), **out)


# --------------------------------------------------------------------- loop + step
def run_loop(exe, sc: scenes.Scene, nsteps, snaps, iters=None, dyn=0):
    nb, ng = sc.nb, sc.ng
    hdr = np.array([nb, ng, nsteps, iters or sc.iterations, dyn, sc.maxc, sc.surface_mode, len(snaps),
                    sc.hash_levels[0], sc.hash_levels[1]], np.int32)
    r = Reader(run(exe, "loop", [hdr, sc.world_params(), sc.surface(), np.array(snaps, np.int32),
                                 sc.bodies, sc.geom_cls, sc.geom_body, sc.geom_pos, sc.geom_R,
                                 sc.geom_dims]))
    snapshots = []
    for _ in snaps:
        step = int(r.take(np.int32, 1)[0])
        nc = int(r.take(np.int32, 1)[0])
        pre = r.take(np.float32, 25 * nb).reshape(nb, 25)
        cb = r.take(np.int32, 2 * nc).reshape(nc, 2)
        cs = r.take(np.float32, 16 * nc).reshape(nc, 16)
        post = r.take(np.float32, 25 * nb).reshape(nb, 25)
        snapshots.append(dict(step=step, pre=pre, cb=cb, cs=cs, post=post))
    traj = r.take(np.float32, nsteps * nb * 7).reshape(nsteps, nb, 7)
    assert r.done()
    return snapshots, traj


def bodies_from_state(state, sc: scenes.Scene):
    """BODY_IN rows (pos q lvel avel mass I) from a BODY_OUT snapshot."""
    b = sc.bodies.copy()
    b[:, 0:3] = state[:, 0:3]
    b[:, 3:7] = state[:, 3:7]
    b[:, 7:10] = state[:, 19:22]
    b[:, 10:13] = state[:, 22:25]
    return b


def run_step(exe, sc, bodies, cb, cs, iters, dyn, stepper, messages=None, dynp=None):
    nb, nc = bodies.shape[0], cb.shape[0]
    hdr = np.array([nb, nc, iters, dyn, stepper], np.int32)
    mode = np.full(nc, sc.surface_mode, np.int32)
    extra = [np.asarray(dynp, np.float32)] if dyn == 2 else []
    r = Reader(run(exe, "step", [hdr, sc.world_params(), *extra, bodies, cb.astype(np.int32), mode, cs], messages))
    ok = int(r.take(np.int32, 1)[0])
    lam = r.take(np.float32, 3 * nc).reshape(nc, 3)
    raw = r.take(np.float32, 12 * nc).reshape(nc, 12)
    post = r.take(np.float32, 25 * nb).reshape(nb, 25)
    assert r.done() and ok == 1
    return lam, raw, post


def gen_steps(exes):
    cases = [
        ("box_stack", scenes.box_stack(seed=0), 1000, [0, 1, 2, 10, 100, 500, 999]),
        ("pile256", scenes.pile(256, seed=3), 300, [40, 80, 150, 299]),
        ("capsule_pile96", scenes.capsule_pile(96, seed=2), 300, [60, 120, 299]),
    ]
    for name, sc, nsteps, snaps in cases:
        snapshots, traj = run_loop(exes["single_noreorder"], sc, nsteps, snaps)
        traj_every = 1 if sc.nb <= 16 else 10
        out = dict(bodies0=sc.bodies, geom_cls=sc.geom_cls, geom_body=sc.geom_body,
                   geom_pos=sc.geom_pos, geom_R=sc.geom_R, geom_dims=sc.geom_dims,
                   params=sc.world_params(), surface=sc.surface(),
                   ints=np.array([sc.iterations, sc.maxc, sc.surface_mode, nsteps], np.int32),
                   traj=traj[::traj_every], traj_every=np.array([traj_every], np.int32),
                   snaps=np.array(snaps, np.int32))
        # the stock reference (random reordering, dynamic iterations) for the same loop
        _, traj_stock = run_loop(exes["single"], sc, nsteps, [], dyn=1)
        out["traj_stock"] = traj_stock[::traj_every]
        for k, s in enumerate(snapshots):
            bodies = bodies_from_state(s["pre"], sc)
            lam, raw, post = run_step(exes["single_noreorder"], sc, bodies, s["cb"], s["cs"],
                                      sc.iterations, 0, 0)
            lam200, _, _ = run_step(exes["single_noreorder"], sc, bodies, s["cb"], s["cs"], 200, 0, 0)
            lamd, _, postd = run_step(exes["double"], sc, bodies, s["cb"], s["cs"], sc.iterations, 0, 1)
            drift = float(np.abs(post[:, 0:3] - s["post"][:, 0:3]).max()) if len(post) else 0.0
            out[f"s{k}_pre"], out[f"s{k}_cb"], out[f"s{k}_cs"] = s["pre"], s["cb"], s["cs"]
            out[f"s{k}_post"] = post
            out[f"s{k}_lambda"], out[f"s{k}_feedback"] = lam, raw
            out[f"s{k}_lambda200"], out[f"s{k}_lambda_dantzig"] = lam200, lamd
            out[f"s{k}_post_dantzig"] = postd
            print(f"{name} step {s['step']}: {len(s['cb'])} contacts, replay drift {drift:.2e}, "
                  f"max|lambda| {np.abs(lam).max() if len(lam) else 0:.3g}")
        np.savez_compressed(os.path.join(HERE, f"step_{name}.npz"), **out)


# two more sets of dynamic iteration parameters (premature exit delta, extra
# factor, extra iteration delta): under the first the solves stop early
# (the box stack after 11 of 20 sweeps), under the second between the regular
# count and twice it (the pile after 47 of 30 + 30)
DYN_SETS = (("dyn2", (30.0, 1.0, 1e9)), ("dyn3", (100.0, 1.0, 1000.0)))


def gen_steps_dyn(exes):
    """The step goldens' snapshots stepped once more by the no-reorder
    reference with its dynamic iteration rule on (quickstep.cpp:1823-1856,
    :3253-3285): at the defaults (premature exit below 1e-8, up to
    `iterations` extra sweeps while an adjustment is >= 1e-2) into
    s{k}_lambda_dyn / s{k}_post_dyn, and with each of DYN_SETS into
    s{k}_lambda_<tag> / s{k}_post_<tag>.  The rule only decides when the sweeps
    stop, so its multipliers equal, to the bit, those of a fixed count of
    sweeps; that count (per contact, the smallest fixed count giving its three
    multipliers; the maximum over contacts is the largest island's) is
    s{k}_sweeps_<tag>.  Adds keys to the existing step_*.npz files."""
    for name in ("box_stack", "pile256", "capsule_pile96"):
        path = os.path.join(HERE, f"step_{name}.npz")
        g = dict(np.load(path))
        sc = {"box_stack": scenes.box_stack(seed=0), "pile256": scenes.pile(256, seed=3),
              "capsule_pile96": scenes.capsule_pile(96, seed=2)}[name]
        iters = int(g["ints"][0])
        for k in range(len(g["snaps"])):
            bodies = bodies_from_state(g[f"s{k}_pre"], sc)
            cb, cs = g[f"s{k}_cb"], g[f"s{k}_cs"]
            fixed = [run_step(exes["single_noreorder"], sc, bodies, cb, cs, n, 0, 0)[0]
                     for n in range(1, 2 * iters + 2)]
            for dyn, tag, dynp in ((1, "dyn", None),) + tuple((2, t, p) for t, p in DYN_SETS):
                lam, _, post = run_step(exes["single_noreorder"], sc, bodies, cb, cs, iters, dyn, 0, dynp=dynp)
                sweeps = np.zeros(len(cb), np.int32)
                for n, ln in enumerate(fixed, start=1):
                    hit = (sweeps == 0) & np.all(ln == lam, axis=1)
                    sweeps[hit] = n
                assert np.all(sweeps > 0), (name, k, tag)
                g[f"s{k}_lambda_{tag}"], g[f"s{k}_post_{tag}"], g[f"s{k}_sweeps_{tag}"] = lam, post, sweeps
                print(f"{name} snapshot {k} ({tag}): stopped after {sweeps.max()} sweeps "
                      f"(fixed count {iters}); max|lambda| {np.abs(lam).max():.3g}")
        for t, p in DYN_SETS:
            g[f"{t}_params"] = np.array(p, np.float32)
        np.savez_compressed(path, **g)


def gen_space_pile(exes):
    """A settled pile (4096 bodies, 200 steps of the oracle, which is bit-exact
    with the reference's loop) and the reference's hash-space pair set on its
    poses: bodies resting slightly below z = 0 in the columns at the container
    corner exercise the reference's unsigned bucket arithmetic."""
    from oracle.port.port import Port
    P = Port()
    sc = scenes.pile(4096, seed=5)
    w = P.world(sc.bodies, sc.world_params(), sc.iterations, dyn=0, reorder=0)
    w.attach_space(sc.geom_cls, sc.geom_body, sc.geom_pos, sc.geom_R, sc.geom_dims, sc.hash_levels, sc.maxc,
                   sc.surface_mode, sc.surface())
    for _ in range(200):
        w.sim_step()
    st = w.state()
    ng, n = sc.ng, sc.nb
    pos = np.zeros((ng, 3), np.float32)
    R = np.zeros((ng, 12), np.float32)
    pos[:n], R[:n] = st[:, 0:3], st[:, 7:19]
    # lower the pile 3 cm so resting bodies reach below z = 0 (negative z cells)
    pos[:n, 2] -= 0.03
    R[n:, [0, 5, 10]] = 1
    r = Reader(run(exes["single"], "space", [np.array([ng, -3, 10], np.int32), sc.geom_cls, pos, R, sc.geom_dims]))
    npairs = int(r.take(np.int32, 1)[0])
    pairs = r.take(np.int32, 2 * npairs).reshape(-1, 2)
    assert r.done()
    np.savez_compressed(os.path.join(HERE, "space_pile.npz"), cls=sc.geom_cls, pos=pos, R=R, dims=sc.geom_dims,
                        body=sc.geom_body, pairs=pairs)
    # pairs whose AABBs overlap but the reference does not report (its bucket
    # arithmetic for negative z near the origin)
    lo, hi = [], []
    for i in range(n):
        d, Rm = sc.geom_dims[i], R[i].reshape(3, 4)[:, :3]
        if sc.geom_cls[i] == scenes.SPHERE:
            r3 = np.full(3, d[0], np.float32)
        else:
            r3 = (np.float32(0.5) * (np.abs(Rm[:, 0] * d[0]) + np.abs(Rm[:, 1] * d[1]) + np.abs(Rm[:, 2] * d[2])))
        lo.append(pos[i] - r3)
        hi.append(pos[i] + r3)
    lo, hi = np.array(lo, np.float32), np.array(hi, np.float32)
    ov = np.all((lo[:, None, :] <= hi[None, :, :]) & (lo[None, :, :] <= hi[:, None, :]), axis=2)
    ii, jj = np.nonzero(np.triu(ov, 1))
    exact = set(zip(ii.tolist(), jj.tolist()))
    ref_bodies = {tuple(p) for p in pairs.tolist() if p[1] < n}
    print(f"space_pile: {ng} geoms, {npairs} reference pairs, {len(exact - ref_bodies)} overlapping pairs the "
          f"reference misses, {len(ref_bodies - exact)} extra")


def gen_joint_scene(exes, sc, name, iters=200, nsteps=240, stepper=False):
    """The reference (no-reorder build) steps a jointed scene without geoms
    (dWorldQuickStep, or dWorldStep with `stepper`): poses per step, then the
    hinge angles and hinge2 steering angles."""
    jt = np.ascontiguousarray(sc.joints, np.float32)
    damp = np.asarray(sc.damping, np.float32)
    buf = run(exes["single_noreorder"], "chain",
              [np.array([sc.nb, len(jt), nsteps, iters, 2 if stepper else 0], np.int32), sc.world_params(),
               sc.bodies.astype(np.float32), jt, damp])
    r = Reader(buf)
    traj = r.take(np.float32, nsteps * sc.nb * 7).reshape(nsteps, sc.nb, 7)
    nh = int(((jt[:, 0] == 2) | (jt[:, 0] == 6)).sum())
    ang = r.take(np.float32, nsteps * nh).reshape(nsteps, nh)
    np.savez_compressed(os.path.join(HERE, name), bodies=sc.bodies, joints=jt, params=sc.world_params(),
                        ints=np.array([iters, nsteps], np.int32), traj=traj, angles=ang, damping=damp)
    print(f"{name}: {sc.nb} bodies, {len(jt)} joints ({nh} with angles), {nsteps} steps")


def gen_hinge2(exes):
    """Vehicles hanging from the environment by a ball joint at the chassis,
    wheels on hinge2 joints (suspension, locked steering, motored axles), no
    geoms: 240 steps of the no-reorder build with 200 iterations."""
    gen_joint_scene(exes, scenes.vehicles(4, seed=21, hang=True), "hinge2.npz")


def gen_chain(exes):
    """Hanging chains of capsules linked by hinge (limited +-60 deg) and ball
    joints, no geoms: 240 steps of the no-reorder build with 200 iterations
    (a converged solve), poses and hinge angles per step."""
    gen_joint_scene(exes, scenes.chains(6, seed=11, nmin=3, nmax=8, hang=True), "chain.npz")


def gen_damped(exes):
    """The hanging chains of chain.npz with world damping (linear 0.02 above
    0.05 m/s, angular 0.05 above 0.1 rad/s) and an angular speed cap of
    1.5 rad/s that the swinging links reach."""
    sc = scenes.chains(6, seed=11, nmin=3, nmax=8, hang=True)
    sc.damping = (0.02, 0.05, 0.05, 0.1, 1.5)
    gen_joint_scene(exes, sc, "damped.npz")


def gen_chain_step(exes):
    """The hanging chains of chain.npz stepped by the reference's dWorldStep
    (Dantzig LCP per island)."""
    gen_joint_scene(exes, scenes.chains(6, seed=11, nmin=3, nmax=8, hang=True), "chain_step.npz", stepper=True)


def gen_step_dantzig32(exes):
    """Adds to every step golden the single-precision reference's dWorldStep
    (Dantzig) multipliers and post-step state of each snapshot, and for both
    precisions whether the reference's LCP solver reported its internal error
    (s <= 0: it then zeroes the multipliers it has not reached, lcp.cpp:1087-
    1096) -- it does on the box stack, whose four coplanar contacts per face
    make the island's matrix nearly singular."""
    cases = [("box_stack", scenes.box_stack(seed=0)), ("pile256", scenes.pile(256, seed=3)),
             ("capsule_pile96", scenes.capsule_pile(96, seed=2))]
    for name, sc in cases:
        path = os.path.join(HERE, f"step_{name}.npz")
        with np.load(path) as z:
            out = {k: z[k] for k in z.files}
        for k in range(len(out["snaps"])):
            bodies = bodies_from_state(out[f"s{k}_pre"], sc)
            m32, m64 = [], []
            lam, _, post = run_step(exes["single_noreorder"], sc, bodies, out[f"s{k}_cb"], out[f"s{k}_cs"],
                                    sc.iterations, 0, 1, m32)
            run_step(exes["double"], sc, bodies, out[f"s{k}_cb"], out[f"s{k}_cs"], sc.iterations, 0, 1, m64)
            out[f"s{k}_lambda_dantzig32"], out[f"s{k}_post_dantzig32"] = lam, post
            err32, err64 = "LCP internal error" in m32[0], "LCP internal error" in m64[0]
            out[f"s{k}_dantzig_lcp_error"] = np.array([err32, err64], np.int32)
            d = np.abs(lam - out[f"s{k}_lambda_dantzig"]).max() / max(1.0, float(np.abs(lam).max()))
            print(f"{name} snapshot {k}: {len(lam)} contacts, single vs double Dantzig lambda {d:.2e}, "
                  f"LCP error single {err32} double {err64}")
        np.savez_compressed(path, **out)


def gen_sleep(exes):
    """Auto-disable in the reference's loop (no-reorder build): two box
    stacks that fall asleep, one struck by a dropped box and woken, for two
    sets of auto-disable parameters (instantaneous velocity over 10 idle
    steps; a 4-sample average over 5 idle steps and 0.05 s): poses and
    dBodyIsEnabled per step."""
    out = {}
    for tag, adis in (("a", (1, 0.15, 0.15, 10, 0.0, 1)), ("b", (1, 0.02, 0.05, 5, 0.05, 4))):
        sc = scenes.sleep_stacks(seed=0, adis=adis)
        nsteps = 300
        hdr = np.array([sc.nb, sc.ng, nsteps, sc.iterations, 0, sc.maxc, sc.surface_mode,
                        sc.hash_levels[0], sc.hash_levels[1]], np.int32)
        r = Reader(run(exes["single_noreorder"], "sleep",
                       [hdr, sc.world_params(), sc.surface(), sc.bodies, sc.geom_cls, sc.geom_body, sc.geom_pos,
                        sc.geom_R, sc.geom_dims, np.asarray(adis, np.float32)]))
        traj = r.take(np.float32, nsteps * sc.nb * 7).reshape(nsteps, sc.nb, 7)
        en = r.take(np.int32, nsteps * sc.nb).reshape(nsteps, sc.nb)
        assert r.done()
        out[f"{tag}_adis"] = np.asarray(adis, np.float32)
        out[f"{tag}_traj"] = traj
        out[f"{tag}_enabled"] = en
        asleep = (en == 0).sum(axis=1)
        print(f"sleep {tag}: asleep bodies at steps 0,10,20,50,80,100,150,200,299: "
              f"{asleep[[0, 10, 20, 50, 80, 100, 150, 200, 299]].tolist()}")
    np.savez_compressed(os.path.join(HERE, "sleep.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("ODE_REFERENCE_DIR"),
                    help="reference source tree (default: $ODE_REFERENCE_DIR)")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not a.ref:
        ap.error("--ref or ODE_REFERENCE_DIR must name the reference source tree")
    exes = build(a.ref)
    if a.only in ("", "colliders"):
        gen_colliders(exes)
    if a.only in ("", "space"):
        gen_space(exes)
    if a.only in ("", "steps"):
        gen_steps(exes)
    if a.only in ("", "space_pile"):
        gen_space_pile(exes)
    if a.only in ("", "chain"):
        gen_chain(exes)
    if a.only in ("", "hinge2"):
        gen_hinge2(exes)
    if a.only in ("", "damped"):
        gen_damped(exes)
    if a.only in ("", "sleep"):
        gen_sleep(exes)
    if a.only in ("", "chain_step"):
        gen_chain_step(exes)
    if a.only in ("", "dantzig32"):
        gen_step_dantzig32(exes)
    if a.only in ("", "steps_dyn"):
        gen_steps_dyn(exes)


if __name__ == "__main__":
    main()
