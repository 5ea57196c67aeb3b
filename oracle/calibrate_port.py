"""Times the CPU port (oracle/slo.cpp, the benchmark's CPU baseline) against
SoftLight's own draw-path sources built by oracle/ref_build.py, on the same
seeded workload with the same thread count: frames alternate between the two,
one warm-up frame each, median of the rest. Needs the reference tree, so it
runs only where oracle/ref_build.py can build (test infrastructure; the
result is recorded in profiles/cpu_calibration.json).

    python oracle/calibrate_port.py <c1|c2|c3|c4> [threads] [frames]
"""
import os
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

# reduced C3 / C4 keep a run within minutes (same generators)
WORKLOADS = {"c1": {}, "c2": {}, "c3": dict(num_tris=500000), "c4": dict(num_draws=64)}


def main():
    import oracle
    import ref_build
    from softlight_gb300 import scenes as S
    from softlight_gb300.api import SLContext, open_library

    name = sys.argv[1]
    threads = int(sys.argv[2]) if len(sys.argv) > 2 else 4
    frames = int(sys.argv[3]) if len(sys.argv) > 3 else 5
    builder = {"c1": S.build_c1, "c2": S.build_c2, "c3": S.build_c3, "c4": S.build_c4}[name]
    lib = open_library(ref_build.build_ref(), "slr_", gpu=False)
    ref = SLContext(lib, "slr_", gpu=False)
    ref.num_threads(threads)
    port = oracle.Context(num_threads=threads)
    sr, sp = builder(ref, **WORKLOADS[name]), builder(port, **WORKLOADS[name])
    sr.render()
    sp.render()
    tr, tp = [], []
    for _ in range(frames):
        t0 = time.perf_counter()
        sr.render()
        tr.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        sp.render()
        tp.append(time.perf_counter() - t0)
    mr, mp = statistics.median(tr), statistics.median(tp)
    print(f"{name} threads={threads} reference {mr * 1000:.1f} ms/frame, port {mp * 1000:.1f} ms/frame, "
          f"port/reference speed {mr / mp:.2f}")


if __name__ == "__main__":
    main()
