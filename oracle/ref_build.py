"""Build recipe of oracle/_ref: SoftLight's own draw-path sources compiled
unmodified from the reference tree against the LightSky compatibility shim in
oracle/ref_shim (the LightSky submodules are empty in the reference tree),
plus oracle/ref_harness.cpp, which exposes them through the same C API as the
CPU oracle (symbol prefix "slr_").

Configuration: no architecture macro is defined, so every #if ladder in the
reference takes its portable branch; -O2 -ffp-contract=off; the context runs
one thread. The library is written to oracle/_ref/libslref.so (git-ignored).
It needs the reference tree, so it is built only where that tree exists; it
is used to validate the CPU oracle and to generate tests/golden fixtures.
"""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libslref.so")
REF = os.environ.get("SOFTLIGHT_REF", "/root/reference/softlight")


def available():
    """Whether the reference tree this recipe compiles is present (it is not
    on machines that only run the tests and the benchmark)."""
    return os.path.isdir(REF)

SOURCES = [
    "SL_BlitCompressedProcessor.cpp", "SL_BlitProcessor.cpp", "SL_ClearProcessor.cpp", "SL_Color.cpp",
    "SL_Context.cpp", "SL_FragmentProcessor.cpp", "SL_Framebuffer.cpp", "SL_Geometry.cpp",
    "SL_IndexBuffer.cpp", "SL_LineProcessor.cpp", "SL_LineRasterizer.cpp", "SL_Mesh.cpp",
    "SL_PipelineState.cpp", "SL_PointProcessor.cpp", "SL_PointRasterizer.cpp", "SL_ProcessorPool.cpp",
    "SL_ShaderProcessor.cpp", "SL_Texture.cpp", "SL_TriProcessor.cpp", "SL_TriRasterizer.cpp",
    "SL_UniformBuffer.cpp", "SL_VertexArray.cpp", "SL_VertexBuffer.cpp", "SL_VertexProcessor.cpp",
    "SL_ViewportState.cpp",
    # scene graph (the caller of the batched draw path)
    "SL_Animation.cpp", "SL_AnimationChannel.cpp", "SL_AnimationKeyList.cpp", "SL_BoundingBox.cpp", "SL_Camera.cpp", "SL_Material.cpp",
    "SL_SceneGraph.cpp", "SL_Transform.cpp",
]

CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-pthread", "-w",
            "-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(REF, "include")]


def _compile(src):
    obj = os.path.join(OUT, "obj", os.path.basename(src) + ".o")
    res = subprocess.run(["g++", *CXXFLAGS, "-c", src, "-o", obj], capture_output=True, text=True)
    return src, obj, res.returncode, res.stderr


def build_ref(force=False):
    """Compile the reference sources + harness into oracle/_ref/libslref.so."""
    if not os.path.isdir(REF):
        raise RuntimeError(f"reference tree not found at {REF}")
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    srcs = [os.path.join(REF, "src", s) for s in SOURCES] + [os.path.join(HERE, "ref_harness.cpp")]
    shim = [os.path.join(dp, f) for dp, _, fs in os.walk(os.path.join(HERE, "ref_shim")) for f in fs]
    newest = max(os.path.getmtime(p) for p in srcs + shim + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        results = list(ex.map(_compile, srcs))
    errors = [(s, e) for s, _, rc, e in results if rc != 0]
    if errors:
        msg = "\n".join(f"== {s}\n{e[:4000]}" for s, e in errors)
        raise RuntimeError(f"reference build failed:\n{msg}")
    objs = [o for _, o, _, _ in results]
    res = subprocess.run(["g++", "-shared", "-pthread", "-o", LIB + ".tmp", *objs], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference link failed:\n{res.stderr[:4000]}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_ref(force=True))
