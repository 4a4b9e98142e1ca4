"""Reference input directories from the seeded generators (command line).

The reference reads a whole case from ``data/*.dat`` (Nmr_start.dat,
Nmr_data.dat, Nmr_grad.dat, Poro.dat, Vx/Vy/Vz.dat, n1_init.dat; the formats
are restated in datfiles.py) and ships none of the large files. This writes a
complete directory from a seed, so that the reference's own executable and
this package's drop-in executable read identical inputs:

    python -m initializator_gb300.gen OUT --preset c1
    python -m initializator_gb300.gen OUT --shape 96 96 64 --geometry grf --sigma 3 \\
        --porosity 0.25 --flow 1e-3 --seed 7 --set n_sequence=9 --set time2=0.05

Presets follow the synthetic workloads (grid, geometry, flow, fluid):
  c1   64^3 sphere pack (r 6, solid 0.35), no flow, rho 10 um/s
  c2   256^3 sphere pack (r 10, solid 0.4), curl-noise flow 1 mm/s
  c3a  384 x 384 x 256 Gaussian random field (sigma 3, porosity 0.25), flow 1 mm/s
  c5   1024 x 1024 x 768 Gaussian random field (sigma 5, porosity 0.2), flow 2 mm/s
       (tens of GB of text in the reference's formats; --device cuda generates it faster)
Every Nmr_data.dat parameter can be set with --set name=value (the field
names of datfiles.NmrData); n_velocity follows --flow unless set explicitly.
--surfrel-water R1 R2 (and --surfrel-oil) writes SurfRel{1,2}<fluid>{X,Y,Z}.dat
face relaxivities (m/s) and switches nSurfRel<fluid> on; --surfrel-spread f
scales each face by a seeded factor in [1 - f, 1 + f].
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import sys

import numpy as np

from . import datfiles, geometry

_WATER = dict(dx=1e-6, dy=1e-6, dz=1e-6, d_water=2.3e-9, t1_water=2.5, t2_water=2.0)

PRESETS = {
    "c1": dict(shape=(64, 64, 64), geometry="spheres", radius=6.0, solid_fraction=0.35, flow=0.0,
               data=dict(_WATER, r1_water=1e-5, r2_water=1e-5)),
    "c2": dict(shape=(256, 256, 256), geometry="spheres", radius=10.0, solid_fraction=0.4, flow=1e-3,
               flow_sigma=4.0, data=dict(_WATER, r1_water=1e-5, r2_water=1e-5)),
    "c3a": dict(shape=(384, 384, 256), geometry="grf", sigma=3.0, porosity=0.25, flow=1e-3, flow_sigma=4.0,
                data=dict(_WATER, r1_water=1e-5, r2_water=1e-5)),
    "c5": dict(shape=(1024, 1024, 768), geometry="grf", sigma=5.0, porosity=0.2, flow=2e-3, flow_sigma=4.0,
               data=dict(_WATER, r1_water=1e-5, r2_water=1e-5)),
}


def _parse_set(items):
    """--set name=value pairs -> {name: value} typed as the NmrData field."""
    types = {f.name: f.type for f in dataclasses.fields(datfiles.NmrData)}
    out = {}
    for item in items:
        name, sep, value = item.partition("=")
        name = name.strip()
        if not sep or name not in types:
            raise SystemExit(f"--set {item!r}: expected name=value with name one of the Nmr_data.dat fields")
        out[name] = int(value) if types[name] in (int, "int") else float(value)
    return out


def build_case(spec, seed=0, device="cpu"):
    """(mask, velocity or None) of a case spec: shape (nx, ny, nz), geometry
    'spheres' (radius, solid_fraction), 'grf' (sigma, porosity) or 'open'
    (every voxel pore), flow (maximum speed, m/s; 0 for none), flow_sigma."""
    nx, ny, nz = spec["shape"]
    shape = (nz, ny, nx)
    kind = spec["geometry"]
    if kind == "spheres":
        mask = geometry.sphere_pack(shape, spec["radius"], spec["solid_fraction"], seed=seed, device=device)
    elif kind == "grf":
        mask = geometry.gaussian_random_field(shape, spec["sigma"], spec["porosity"], seed=seed, device=device)
    elif kind == "open":
        mask = np.ones(shape, np.uint8)
    else:
        raise ValueError(f"unknown geometry {kind!r}")
    vel = None
    if spec.get("flow", 0.0) > 0.0:
        vel = geometry.curl_velocity(mask, spec.get("flow_sigma", 4.0), spec["flow"], seed=seed + 1, device=device)
    return mask, vel


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m initializator_gb300.gen",
                                 description="write a reference input directory (data/*.dat) from a seed")
    ap.add_argument("out", help="case directory (data/ is created inside it)")
    ap.add_argument("--preset", choices=sorted(PRESETS))
    ap.add_argument("--shape", nargs=3, type=int, metavar=("NX", "NY", "NZ"))
    ap.add_argument("--geometry", choices=["spheres", "grf", "open"])
    ap.add_argument("--radius", type=float, help="sphere radius in voxels (spheres)")
    ap.add_argument("--solid-fraction", type=float, help="solid volume fraction (spheres)")
    ap.add_argument("--sigma", type=float, help="smoothing length in voxels (grf)")
    ap.add_argument("--porosity", type=float, help="pore volume fraction (grf)")
    ap.add_argument("--flow", type=float, help="maximum flow speed in m/s; 0 writes no velocity files")
    ap.add_argument("--flow-sigma", type=float, help="smoothing length of the flow's vector potential (voxels)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--grad", type=float, nargs="+", default=[0.0], help="Nmr_grad.dat values (T/m)")
    ap.add_argument("--n1", type=float, help="uniform phase-1 concentration for two components (n1_init.dat)")
    ap.add_argument("--n1-random", type=float, nargs=2, metavar=("LOW", "HIGH"),
                    help="seeded uniform phase-1 concentration in [LOW, HIGH) (n1_init.dat)")
    ap.add_argument("--surfrel-water", type=float, nargs=2, metavar=("R1", "R2"),
                    help="face relaxivities of water (SurfRel1WaterX.dat ... SurfRel2WaterZ.dat), m/s")
    ap.add_argument("--surfrel-oil", type=float, nargs=2, metavar=("R1", "R2"),
                    help="face relaxivities of oil (SurfRel1OilX.dat ... SurfRel2OilZ.dat), m/s")
    ap.add_argument("--surfrel-spread", type=float, default=0.0,
                    help="seeded relative spread of the face relaxivities")
    ap.add_argument("--set", action="append", default=[], metavar="NAME=VALUE",
                    help="an Nmr_data.dat parameter (datfiles.NmrData field name)")
    ap.add_argument("--device", default="cpu", help="torch device for the generators")
    args = ap.parse_args(argv)

    spec = dict(PRESETS[args.preset]) if args.preset else {"data": {}}
    spec["data"] = dict(spec.get("data", {}))
    for key in ("shape", "geometry", "radius", "solid_fraction", "sigma", "porosity", "flow", "flow_sigma"):
        v = getattr(args, key)
        if v is not None:
            spec[key] = tuple(v) if key == "shape" else v
    if "shape" not in spec or "geometry" not in spec:
        ap.error("give --preset or both --shape and --geometry")
    need = {"spheres": ("radius", "solid_fraction"), "grf": ("sigma", "porosity"), "open": ()}[spec["geometry"]]
    missing = [k for k in need if k not in spec]
    if missing:
        ap.error(f"geometry {spec['geometry']} needs " + ", ".join("--" + k.replace("_", "-") for k in missing))

    mask, vel = build_case(spec, seed=args.seed, device=args.device)
    data_kw = dict(spec["data"])
    data_kw["n_velocity"] = 1 if vel is not None else 0
    if args.surfrel_water is not None:
        data_kw["n_surf_rel_water"] = 1
    if args.surfrel_oil is not None:
        data_kw["n_surf_rel_oil"] = 1
    data_kw.update(_parse_set(args.set))
    data = datfiles.NmrData(**data_kw)
    if data.n_velocity == 1 and vel is None:
        ap.error("n_velocity=1 needs --flow > 0")
    n1 = None
    if args.n1 is not None:
        n1 = np.full(mask.shape, args.n1, np.float32)
    elif args.n1_random is not None:
        lo, hi = args.n1_random
        n1 = np.random.default_rng(args.seed + 2).uniform(lo, hi, mask.shape).astype(np.float32)
    if data.n_components == 2 and n1 is None:
        ap.error("n_components=2 needs --n1 or --n1-random")
    if args.surfrel_spread < 0.0 or args.surfrel_spread >= 1.0:
        ap.error("--surfrel-spread must be in [0, 1)")
    surfrel = {}
    rng = np.random.default_rng(args.seed + 3)
    nz_, ny_, nx_ = mask.shape
    faces = ((nz_, ny_, nx_ + 1), (nz_, ny_ + 1, nx_), (nz_ + 1, ny_, nx_))
    for fluid, vals, flag in (("Water", args.surfrel_water, data.n_surf_rel_water),
                              ("Oil", args.surfrel_oil, data.n_surf_rel_oil)):
        if flag == 1 and vals is None:
            ap.error(f"nSurfRel{fluid} = 1 needs --surfrel-{fluid.lower()}")
        if vals is None:
            continue
        for n, r in zip("12", vals):
            s = args.surfrel_spread
            surfrel[n + fluid] = tuple(r * (1.0 + rng.uniform(-s, s, f)) if s > 0 else np.full(f, r) for f in faces)

    datfiles.write_case(args.out, data, mask, vel=None if data.n_velocity != 1 else vel, grads=tuple(args.grad),
                        surfrel=surfrel, n1=n1)
    nx, ny, nz = spec["shape"]
    summary = {"dir": os.path.join(args.out, "data"), "shape": [nx, ny, nz], "geometry": spec["geometry"],
               "seed": args.seed, "porosity": float(mask.mean()), "velocity": data.n_velocity == 1,
               "two_components": data.n_components == 2, "surfrel": sorted(surfrel)}
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    sys.exit(main())
