"""Generate tests/golden/reference_pins.json from the reference's own code
(run where the reference tree is present; $ZGL_REFERENCE_TREE names it).

* The PackedBVH of the traversal soups (1M / 4M / 16M triangles) as the
  reference's BVH::build() makes it (src/accelerator/BVH.cpp compiled by
  oracle/build_oracle.py behind stand-in headers), by SHA-256.
* Path-tracer frames rendered by the reference's path_integ_naive.glsl and
  light / triple films rendered by light_path_integ.glsl and
  triple_path_pass_{pt,lpt}.glsl, each compiled as C++ by
  oracle/glsl_to_cpp.py (frames by SHA-256, films whole).
* bvhHit / bvhTest results of the reference shader on a 60k soup.

The cases are defined in tests/reference_pin_cases.py.  GPU tests compare the
CUDA path with this file on machines that have no reference tree.
"""
from __future__ import annotations

import base64
import json
import sys
import time
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from tests.reference_pin_cases import (FILM_CASES, FRAME_CASES, SOUPS, TRACE_CASE, frame_rgb,  # noqa: E402
                                       mixed_rays, sha256)
from zillumgl_gb300.scene import Scene  # noqa: E402
from zillumgl_gb300.synthetic import TRAVERSAL_SEEDS, triangle_soup  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_pins.json"


def encode(a: np.ndarray) -> str:
    return base64.b64encode(zlib.compress(np.ascontiguousarray(a, np.float32).tobytes(), 9)).decode()


def decode(s: str, shape) -> np.ndarray:
    return np.frombuffer(zlib.decompress(base64.b64decode(s)), np.float32).reshape(shape)


def frame_pin(name):
    make, params, passes = FRAME_CASES[name]
    d = make()
    sc = Scene(d, host_only=True)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    W, H = d.film
    rgb = orc.glsl_render_pt(np.arange(W * H), passes).reshape(H, W, 3)
    sc.close()
    return {"film": [W, H], "passes": passes, "sha256": sha256(frame_rgb(rgb)), "mean": float(rgb.mean())}


def film_pin(name):
    kind, make, params, passes, blocks, loops = FILM_CASES[name]
    d = make()
    sc = Scene(d, host_only=True)
    orc = oracle.OracleScene(d, sc.export("sobol"), params)
    if kind == "light":
        film = orc.glsl_render_lt(passes, blocks=blocks)
    else:
        film = orc.glsl_render_triple(passes, blocks=blocks, loops=loops)
    sc.close()
    return {"shape": list(film.shape), "film": encode(film), "sum": float(film.sum())}


def soup_pin(n):
    v, idx = triangle_soup(n, TRAVERSAL_SEEDS[n])
    bounds, hit = oracle.ref_bvh_build(v, idx)
    return {"triangles": n, "seed": TRAVERSAL_SEEDS[n], "nodes": int(bounds.shape[0]), "sha256": sha256(bounds, hit)}


def trace_pin():
    name, ntri, seed, nray, rseed = TRACE_CASE
    v, idx = triangle_soup(ntri, seed)
    bounds, hit = oracle.ref_bvh_build(v, idx)
    o, d = mixed_rays(np.random.default_rng(rseed), nray)
    hid, ht = oracle.glsl_trace(bounds, hit, v, idx, o, d)
    tmax = np.random.default_rng(rseed + 1).random(nray).astype(np.float32)
    occ, _ = oracle.glsl_trace(bounds, hit, v, idx, o, d, tmax=tmax)
    return {"bvh_sha256": sha256(bounds, hit), "closest_sha256": sha256(hid, ht), "any_sha256": sha256(occ),
            "hits": int((hid >= 0).sum()), "occluded": int(occ.sum())}


def main() -> int:
    if oracle.ref_lib() is None or oracle.glsl_lib() is None:
        print("reference tree not present; nothing generated")
        return 1
    out = {"frames": {}, "films": {}, "soups": {}, "trace": {}}
    for name in FRAME_CASES:
        t = time.time()
        out["frames"][name] = frame_pin(name)
        print(f"frame {name}: {time.time() - t:.1f}s", flush=True)
    for name in FILM_CASES:
        out["films"][name] = film_pin(name)
        print(f"film {name}", flush=True)
    out["trace"][TRACE_CASE[0]] = trace_pin()
    for name, n in SOUPS.items():
        t = time.time()
        out["soups"][name] = soup_pin(n)
        print(f"soup {name}: {time.time() - t:.1f}s", flush=True)
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
