"""Regenerates the committed fixtures of this folder.

0. mesh_torus.npz: the reference's triangle mesh public/model/torus.obj.
1. cdm_*.npz: the reference's boundary assets public/model/torus.cdm and
   public/model/domain_boundary.cdm (20^3 cubic volume maps over the unit
   cube), parsed exactly as BoundaryModel.setData does
   (src/simulator/boundary/volumeMap.ts:23-39) and stored as float32 arrays.
   Needs the environment variable REFERENCE_ROOT set to a checkout of the
   reference (the script refuses to guess a path).
2. oracle_*.npz: outputs of the CPU restatement (oracle/) on small seeded
   inputs, kept as regression vectors for the restatement itself.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE_ROOT = os.environ.get("REFERENCE_ROOT")


def _reference_root():
    if not REFERENCE_ROOT:
        raise SystemExit("set REFERENCE_ROOT to the reference checkout (or pass --oracle-only)")
    return REFERENCE_ROOT


def parse_cdm_text(text):
    lines = text.split("\n")
    res = [int(float(t)) for t in lines[0].split()]
    # the reference drops the last token of lines 2 and 4 (a trailing space)
    sdf = np.array([float(t) for t in lines[2].split(" ")[:-1]], dtype=np.float32)
    vol = np.array([float(t) for t in lines[4].split(" ")[:-1]], dtype=np.float32)
    return np.array(res, dtype=np.uint32), sdf, vol, lines[1].strip(), lines[3].strip()


def make_cdm():
    for name in ("torus", "domain_boundary"):
        path = os.path.join(_reference_root(), "public", "model", name + ".cdm")
        with open(path) as f:
            res, sdf, vol, n1, n2 = parse_cdm_text(f.read())
        assert int(n1) == sdf.size and int(n2) == vol.size
        np.savez_compressed(os.path.join(HERE, "cdm_%s.npz" % name), res=res, sdf=sdf, vol=vol)
        print(name, res, sdf.size)


def make_meshes():
    """mesh_torus.npz: the reference's public/model/torus.obj (400 vertices,
    800 triangles) as float32 vertices and uint32 triangles."""
    sys.path.insert(0, os.path.join(REPO, "webgpu-fluid-simulation_gb300"))
    from pbf_gb300 import scenes
    with open(os.path.join(_reference_root(), "public", "model", "torus.obj")) as f:
        v, t = scenes.parse_obj(f.read())
    np.savez_compressed(os.path.join(HERE, "mesh_torus.npz"), vertices=v, triangles=t)
    print("torus mesh", v.shape, t.shape)


def make_oracle():
    sys.path.insert(0, REPO)
    sys.path.insert(0, os.path.join(REPO, "webgpu-fluid-simulation_gb300"))
    from oracle import oracle as O
    from pbf_gb300 import scenes
    # neighbour search on a clumped 128^3-cell case (4096 particles)
    cfg, pts = scenes.neighbor_case(4096, "clumps", seed=7, dim=128)
    ns = O.neighbor_search(cfg, pts, lists=False)
    np.savez_compressed(os.path.join(HERE, "oracle_ns_clumps4096.npz"), pts=pts, keys=ns["keys"],
                        cell_count=ns["cell_count"], cell_offset=ns["cell_offset"], order=ns["order"],
                        rank=ns["rank"])
    # one substep of a small reference-constants scene (2197 particles)
    sc = scenes.reference_scene("cube_small")
    o = O.Oracle(sc.config, 32)
    o.set_particles(sc.particles)
    o.substep(1)
    np.savez_compressed(os.path.join(HERE, "oracle_step_cube2197.npz"), pts=sc.particles,
                        position=o.field(0).astype(np.float32), velocity=o.field(1).astype(np.float32),
                        acceleration=o.field(2).astype(np.float32), lam=o.field(4).astype(np.float32))
    print("oracle fixtures written")


if __name__ == "__main__":
    if "--oracle-only" not in sys.argv:
        make_meshes()
        make_cdm()
    make_oracle()
