"""Generates the golden fixtures in this folder from SoftLight's own draw-path
sources: oracle/_ref/libslref.so, built by oracle/ref_build.py from the
reference tree (compiled unmodified against the LightSky shim in
oracle/ref_shim, portable branches, one thread).

Each fixture is <name>.npz holding the colour and depth attachments after
one frame of a seeded workload (tests/golden_scenes.py), plus SHA-256 digests
of both arrays with every NaN replaced by one canonical NaN (x86 and aarch64
produce different NaN payloads); blits.npz holds the results of the blit
cases of tests/golden_scenes.py (blit_cases). Run from the repository root:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))


def canonical(a):
    a = np.ascontiguousarray(a).copy()
    if a.dtype.kind == "f":
        a[np.isnan(a)] = a.dtype.type("nan")
    return a


def digest(a):
    return hashlib.sha256(canonical(a).tobytes()).hexdigest()


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_build
    from softlight_gb300.api import SLContext, open_library
    import golden_scenes as G

    lib = open_library(ref_build.build_ref(), "slr_", gpu=False)
    index = {}
    for name, (builder, kw) in G.SCENES.items():
        ctx = SLContext(lib, "slr_", gpu=False)
        scene = builder(ctx, **kw)
        scene.render()
        color, depth = scene.read_color(), scene.read_depth()
        extra = {f"color{k}": scene.read_color(k) for k in range(1, len(scene.attachments))}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), color=color, depth=depth, **extra)
        index[name] = {"color_sha256": digest(color), "depth_sha256": digest(depth),
                       "shape": list(color.shape), "covered": int((depth < scene.clear_depth).sum())}
        ctx.close()
        print(name, index[name]["covered"])
    with open(os.path.join(HERE, "index.json"), "w") as fh:
        json.dump(index, fh, indent=1, sort_keys=True)

    # blits (SL_Context::blit) of rendered attachments
    ctx = SLContext(lib, "slr_", gpu=False)
    blits = G.blit_cases(ctx)
    ctx.close()
    np.savez_compressed(os.path.join(HERE, "blits.npz"), **blits)
    print("blits", sorted(blits))

    # the scene graph: update + mesh-node traversal over three frames
    graph = G.scene_graph_cases(lambda: SLContext(lib, "slr_", gpu=False))
    np.savez_compressed(os.path.join(HERE, "scene_graph.npz"), **graph)
    print("scene_graph", sorted(graph))


if __name__ == "__main__":
    main()
