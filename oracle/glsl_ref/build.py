"""Builds oracle/_ref/librgdn_refshaders.so: the reference's own A-SVGF and tonemapping compute
shaders, from their GLSL sources under the reference checkout, run on the CPU (test
infrastructure; nothing of the product links it).

Recipe, per shader:
  1. copy the reference's Source/Shaders headers and Source/Generated/ShaderCommonGLSL.h into
     oracle/_ref/stage/ without their #version / #extension lines, which no C preprocessor reads;
  2. run the C preprocessor over the shader (includes, #if, macros): flat GLSL;
  3. rewrite the flat GLSL as C++ for oracle/glsl_ref/glsl.h, mechanically:
     - layout-qualified images and samplers -> GLSL_IMAGE / GLSL_SAMPLER declarations; uniform and
       buffer blocks -> their members as namespace-scope variables; the local size -> a constant;
       specialisation constants -> constants fixed per build (one build per value used);
     - multi-component swizzles -> .swz<i...>() (read) or .swzw<i...>() (assigned to);
     - float literals -> float (f suffix); T[n](...) array constructors -> { ... };
     - out / inout parameters -> references; shared -> static; main -> shader_main;
  4. compile each shader (and each specialisation) as its own namespace and translation unit,
     with extern "C" entry points: dispatch, the global uniform from rgdn_frame_params, the
     tonemapping buffer;
  5. link with glsl_rt.cpp and planes.cpp into oracle/_ref/librgdn_refshaders.so.
The reference's sources are read where they lie and are not copied into the repository; the
staged and rewritten files live under oracle/_ref/, which git ignores.

Usage: python oracle/glsl_ref/build.py [--reference DIR]
"""
from __future__ import annotations

import argparse
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

# where the reference checkout lies on the machine that builds the checker (the GPU machines have
# none: there the committed vectors stand in for it)
REFERENCE = "/root/reference"

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "librgdn_refshaders.so")

# shader -> {specialisation constant: values built}
SHADERS = {
    "CmASVGFGradientAtrous.comp": {"atrousIteration": [0, 1, 2, 3]},
    "CmSVGFTemporalAccumulation.comp": {},
    "CmAntiFirefly.comp": {},
    "CmSVGFEstimateVariance.comp": {},
    "CmSVGFAtrous_Iter0.comp": {},
    "CmSVGFAtrous.comp": {"atrousIteration": [1, 2, 3, 4, 5]},
    "CmLuminanceHistogram.comp": {},
    "CmLuminanceAvg.comp": {},
    "CmBloomDownsample.comp": {"stepIndex": list(range(8))},
    "CmBloomUpsample.comp": {"stepIndex": list(range(8))},
    # written by gradient_samples_source() from RtGradients.rgen
    "RtGradients_main.comp": {},
    "CmCheckerboard.comp": {},
    "CmPrepareFinal.comp": {},
    "CmBloomApply.comp": {"isSourcePing": [1]},
    "CmVolumetricProcess.comp": {},
    "CmScatterAccum.comp": {},
}

# rgdn_volumetric_params fields that ShGlobalUniform has under the same name (Volumetric's
# uniform inputs of CmVolumetricProcess.comp and CmScatterAccum.comp)
VOLUME_COPY = ["invView", "invProjection", "volumeViewProj", "cameraPosition", "volumeCameraNear",
               "volumeCameraFar", "volumeAmbient", "volumeScattering", "volumeEnableType", "frameId"]

# rgdn_final_params fields that ShGlobalUniform has under the same name (ImageComposition's
# uniform inputs of CmPrepareFinal.comp)
FINAL_COPY = ["luminanceWhitePoint", "emissionMaxScreenColor", "bloomEmissionMultiplier", "bloomThreshold",
              "lightmapScreenCoverage"]

# rgdn_bloom_params fields that ShGlobalUniform has under the same name (Bloom::Apply's uniform
# inputs of CmBloomApply.comp; the lens-dirt term, which this path leaves out, is set to 0)
BLOOM_COPY = ["bloomIntensity"]

# RtGradients.rgen is a ray-generation shader: its main() selects each stratum's sample, tests it,
# and turns the forward-projected luminance into the temporal gradient; only the forward
# projection itself traces rays (re-shading the previous frame's surface with this frame's
# lights). That part is this project's boundary input RGDN_FB_GRADIENT_RESHADED (the luminance
# pair at the previous frame's shading pixel), so the build replaces the statements that compute
# forwardProjectedLuminance with a load of that input and runs the rest of main() as written, one
# invocation per launch index (gl_LaunchIDEXT), over PathTracer::CalculateGradientsSamples's
# ceil(width / 3) x ceil(height / 3) launch.
GRADIENT_PREAMBLE = """#define DESC_SET_FRAMEBUFFERS 0
#define DESC_SET_GLOBAL_UNIFORM 1
#include "ShaderCommonGLSLFunc.h"
layout(local_size_x = 1, local_size_y = 1, local_size_z = 1) in;
layout(set = DESC_SET_FRAMEBUFFERS, binding = 1000, rg32f) uniform image2D framebufGradientReshaded;
#define gl_LaunchIDEXT gl_GlobalInvocationID
"""
GRADIENT_FORWARD = "vec2 forwardProjectedLuminance = imageLoad(framebufGradientReshaded, prevShadingPix).xy;"


def gradient_samples_source(ref: str) -> str:
    """RtGradients.rgen's main() (from its GRADIENT_ESTIMATION_ENABLED block) behind
    GRADIENT_PREAMBLE, with the forward projection replaced by GRADIENT_FORWARD. Every anchor must
    be found exactly once, so a changed shader fails the build instead of building something else."""
    with open(os.path.join(ref, "Source", "Shaders", "RtGradients.rgen"), encoding="utf-8") as f:
        src = f.read()

    def once(pat: str, text: str) -> re.Match:
        ms = list(re.finditer(pat, text))
        if len(ms) != 1:
            raise RuntimeError(f"RtGradients.rgen: {pat!r} found {len(ms)} times")
        return ms[0]

    body = src[once(r"#if\s+GRADIENT_ESTIMATION_ENABLED\b", src).start():]
    start = once(r"const\s+uint\s+oldSeed\s*=", body).start()
    once(r"vec2\s+forwardProjectedLuminance\s*=\s*vec2\(\s*0\.0\s*\)\s*;", body[start:])
    m = once(r"if\s*\(\s*matchedSurface\s*\)\s*\{", body[start:])
    k, depth = start + m.end(), 1
    while depth:
        depth += {"{": 1, "}": -1}.get(body[k], 0)
        k += 1
    return GRADIENT_PREAMBLE + body[:start] + GRADIENT_FORWARD + body[k:]

# rgdn_frame_params fields that ShGlobalUniform has under the same name
UNIFORM_COPY = ["view", "viewPrev", "projection", "projectionPrev", "cameraPosition", "cameraPositionPrev",
                "timeDelta", "minLogLuminance", "maxLogLuminance", "stopEyeAdaptation", "gradientMultDiffuse",
                "gradientMultIndirect", "gradientMultSpecular", "antiFireflyEnabled", "lightmapScreenCoverage",
                "debugShowFlags", "frameId"]

SWZ = {c: i for i, c in enumerate("xyzw")}
SWZ.update({c: i for i, c in enumerate("rgba")})
SWZ.update({c: i for i, c in enumerate("stpq")})


def stage(ref: str) -> str:
    st = os.path.join(OUT, "stage")
    if os.path.isdir(st):
        shutil.rmtree(st)
    os.makedirs(st)
    srcs = []   # (source path, path under the staging directory)
    shaders = os.path.join(ref, "Source", "Shaders")
    for dirpath, _, names in os.walk(shaders):
        for n in names:
            if n.endswith((".h", ".inl", ".comp")):
                p = os.path.join(dirpath, n)
                srcs.append((p, os.path.relpath(p, shaders)))
    srcs.append((os.path.join(ref, "Source", "Generated", "ShaderCommonGLSL.h"), "ShaderCommonGLSL.h"))
    for src, rel in srcs:
        with open(src, encoding="utf-8", errors="replace") as f:
            lines = [ln for ln in f if not re.match(r"\s*#\s*(version|extension)\b", ln)]
        dst = os.path.join(st, rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        with open(dst, "w") as f:
            f.writelines(lines)
    with open(os.path.join(st, "RtGradients_main.comp"), "w") as f:
        f.write(gradient_samples_source(ref))
    return st


def preprocess(st: str, shader: str) -> str:
    r = subprocess.run(["cpp", "-P", "-undef", "-nostdinc", "-x", "c", "-I", st, os.path.join(st, shader)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cpp {shader}:\n{r.stderr}")
    return r.stdout


def matching_paren(s: str, i: int) -> int:
    """Index of the parenthesis closing the one at s[i]."""
    depth = 0
    for k in range(i, len(s)):
        if s[k] == "(":
            depth += 1
        elif s[k] == ")":
            depth -= 1
            if depth == 0:
                return k
    raise ValueError("unbalanced parentheses")


def layout_args(text: str) -> dict:
    out = {}
    for part in text.split(","):
        part = part.strip()
        if "=" in part:
            k, v = part.split("=", 1)
            out[k.strip()] = v.strip().strip("()").strip()
        elif part:
            out[part] = None
    return out


def rewrite(flat: str, spec: dict) -> tuple[str, dict]:
    info = {"local": None, "uniform": False, "tonemapping": False, "barrier": False}
    s = flat

    # --- layout-qualified declarations -------------------------------------------------
    out, pos = [], 0
    quals = r"(?:(?:readonly|writeonly|coherent|restrict|volatile)\s+)*"
    for m in re.finditer(r"\blayout\s*\(", s):
        if m.start() < pos:
            continue
        out.append(s[pos:m.start()])
        close = matching_paren(s, m.end() - 1)
        args = layout_args(s[m.end():close])
        rest = s[close + 1:]
        # local size
        mm = re.match(r"\s*in\s*;", rest)
        if mm and "local_size_x" in args:
            info["local"] = tuple(int(args.get(k, "1") or 1) for k in ("local_size_x", "local_size_y", "local_size_z"))
            pos = close + 1 + mm.end()
            continue
        # specialisation constant, fixed per build
        mm = re.match(r"\s*const\s+(\w+)\s+(\w+)\s*=\s*([^;]+);", rest)
        if mm and "constant_id" in args:
            name = mm.group(2)
            if name not in spec:
                raise RuntimeError(f"specialisation constant {name} without a build value")
            out.append(f"static const {mm.group(1)} {name} = {spec[name]};")
            pos = close + 1 + mm.end()
            continue
        # image / sampler
        mm = re.match(r"\s*" + quals + r"uniform\s+" + quals +
                      r"([iu]?)(image2D|sampler2D|image3D|sampler3D|texture2DArray)\s+(\w+)\s*;", rest)
        if mm:
            typ, name = mm.group(1) + mm.group(2), mm.group(3)
            if mm.group(2) in ("image2D", "image3D"):
                fmt = [k for k, v in args.items() if v is None]
                if len(fmt) != 1:
                    raise RuntimeError(f"image {name}: format not found in layout({args})")
                out.append(f"GLSL_IMAGE({typ}, {name}, {fmt[0]});")
            else:
                out.append(f"GLSL_SAMPLER({typ}, {name});")
            pos = close + 1 + mm.end()
            continue
        # unsized array of samplers (the texture table): every element unbound
        mm = re.match(r"\s*" + quals + r"uniform\s+" + quals + r"(sampler2D)\s+(\w+)\s*\[\s*\]\s*;", rest)
        if mm:
            out.append(f"static glsl::SamplerTable {mm.group(2)};")
            pos = close + 1 + mm.end()
            continue
        # uniform / buffer block
        mm = re.match(r"\s*" + quals + r"(uniform|buffer)\s+" + quals + r"(\w+)\s*\{", rest)
        if mm:
            body_start = close + 1 + mm.end()
            depth, k = 1, body_start
            while depth:
                depth += {"{": 1, "}": -1}.get(s[k], 0)
                k += 1
            body = s[body_start:k - 1]
            tail = re.match(r"\s*(\w*)\s*;", s[k:])
            inst = tail.group(1)
            if inst:
                out.append(f"static struct {mm.group(2)} {{{body}}} {inst};")
            else:
                for decl in [d.strip() for d in body.split(";") if d.strip()]:
                    out.append(f"static {decl};")
                    if re.search(r"\bglobalUniform\b", decl):
                        info["uniform"] = True
                    if re.search(r"\btonemapping\b", decl):
                        info["tonemapping"] = True
            pos = k + tail.end()
            continue
        raise RuntimeError(f"unhandled layout({s[m.end():close]}): {rest[:80]!r}")
    out.append(s[pos:])
    s = "".join(out)

    # --- qualifiers and keywords ---------------------------------------------------------
    s = re.sub(r"\b(readonly|writeonly|coherent|restrict|highp|mediump|lowp|precise|flat|noperspective)\b", "", s)
    s = re.sub(r"\bshared\b", "static", s)
    s = re.sub(r"\b(inout|out)\s+((?:const\s+)?\w+)\s+(\w+)", r"\2 &\3", s)
    s = re.sub(r"\bin\s+((?:const\s+)?\w+)\s+(\w+)\s*([,)])", r"\1 \2\3", s)
    s = re.sub(r"\bvoid\s+main\s*\(", "void shader_main(", s)
    info["barrier"] = bool(re.search(r"\b(barrier|groupMemoryBarrier|memoryBarrierShared)\s*\(", s))

    # --- array constructors T[n](...) -> { ... } ------------------------------------------
    while True:
        m = re.search(r"\b\w+\s*\[\s*\w*\s*\]\s*\(", s)
        if not m:
            break
        close = matching_paren(s, m.end() - 1)
        s = s[:m.start()] + "{" + s[m.end():close] + "}" + s[close + 1:]

    # --- swizzles --------------------------------------------------------------------------
    def swz(m: re.Match) -> str:
        comps = m.group(1)
        idx = ",".join(str(SWZ[c]) for c in comps)
        after = s_now[m.end():m.end() + 8]
        write = re.match(r"\s*(=(?!=)|\+=|-=|\*=|/=)", after) is not None
        return f".{'swzw' if write else 'swz'}<{idx}>()"

    s_now = s
    s = re.sub(r"\.([xyzw]{2,4}|[rgba]{2,4}|[stpq]{2,4})\b(?!\s*\()", lambda m: swz(m), s_now)

    # --- float literals -> float ------------------------------------------------------------
    s = re.sub(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])", r"\1f", s)
    return s, info


def translation_unit(shader: str, body: str, info: dict, tag: str) -> str:
    ns = "sh_" + tag
    lx, ly, lz = info["local"]
    lines = ['#include "glsl.h"', '#include "rgdn.h"', f"namespace {ns} {{", "using namespace glsl;", body,
             f"static const glsl::uvec3 kLocal({lx}u, {ly}u, {lz}u);", "}", 'extern "C" {',
             f"void ref_{tag}_dispatch(unsigned gx, unsigned gy) {{ glsl::dispatch({ns}::shader_main, "
             f"glsl::uvec3(gx, gy, 1u), {ns}::kLocal, {'true' if info['barrier'] else 'false'}); }}",
             f"void ref_{tag}_local(unsigned* out) {{ out[0] = {lx}; out[1] = {ly}; out[2] = {lz}; }}"]
    if info["uniform"]:
        sets = [f"std::memcpy(&u.{f}, &p->{f}, sizeof(p->{f}));" for f in UNIFORM_COPY]
        lines.append(f"void ref_{tag}_set_uniform(const rgdn_frame_params* p, float rw, float rh) {{ "
                     f"auto& u = {ns}::globalUniform; {' '.join(sets)} u.renderWidth = rw; u.renderHeight = rh; }}")
        sets = [f"std::memcpy(&u.{f}, &p->{f}, sizeof(p->{f}));" for f in FINAL_COPY]
        lines.append(f"void ref_{tag}_set_final(const rgdn_final_params* p) {{ "
                     f"auto& u = {ns}::globalUniform; {' '.join(sets)} }}")
        if re.search(r"\blensDirtIntensity\b", body):
            sets = [f"std::memcpy(&u.{f}, &p->{f}, sizeof(p->{f}));" for f in BLOOM_COPY]
            lines.append(f"void ref_{tag}_set_bloom(const rgdn_bloom_params* p) {{ "
                         f"auto& u = {ns}::globalUniform; {' '.join(sets)} u.lensDirtIntensity = 0.0f; }}")
        sets = [f"std::memcpy(&u.{f}, &p->{f}, sizeof(p->{f}));" for f in VOLUME_COPY]
        lines.append(f"void ref_{tag}_set_volumetric(const rgdn_volumetric_params* p) {{ "
                     f"auto& u = {ns}::globalUniform; {' '.join(sets)} }}")
    if re.search(r"\}\s*push\s*;", body):
        # the push-constant block
        lines.append(f"void* ref_{tag}_push() {{ return &{ns}::push; }}")
    if info["tonemapping"]:
        lines.append(f"void* ref_{tag}_tonemapping() {{ return &{ns}::tonemapping; }}")
    if re.search(r"\bstatic\s+uvec4\s+g_lpmParams\s*\[", body):
        # the LPM control block (LpmParams_BT), filled from ref_lpm_setup
        lines.append(f"void* ref_{tag}_lpm() {{ return &{ns}::g_lpmParams; }}")
    lines.append("}")
    return "\n".join(lines) + "\n"


def build(ref: str, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    st = stage(ref)
    src_dir = os.path.join(OUT, "src")
    os.makedirs(src_dir, exist_ok=True)
    units = []
    for shader, specs in SHADERS.items():
        flat = preprocess(st, shader)
        base = shader.split(".")[0]
        combos = [{}]
        for k, vals in specs.items():
            combos = [dict(c, **{k: v}) for c in combos for v in vals]
        for c in combos:
            tag = base + "".join(f"_{v}" for v in c.values())
            body, info = rewrite(flat, c)
            path = os.path.join(src_dir, tag + ".cpp")
            with open(path, "w") as f:
                f.write(translation_unit(shader, body, info, tag))
            units.append(path)
    flags = ["g++", "-std=c++17", "-O1", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w",
             "-I", HERE, "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ref, "Source", "Shaders", "LPM")]
    objs = []

    def cc(src):
        obj = os.path.join(OUT, "obj", os.path.basename(src).replace(".cpp", ".o"))
        os.makedirs(os.path.dirname(obj), exist_ok=True)
        r = subprocess.run(flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile {src}:\n{r.stderr[-6000:]}")
        return obj

    srcs = units + [os.path.join(HERE, "glsl_rt.cpp"), os.path.join(HERE, "lpm_setup_ref.cpp")]
    with ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(cc, srcs))
    r = subprocess.run(["g++", "-shared", "-o", LIB] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=REFERENCE)
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    if not os.path.isdir(os.path.join(a.reference, "Source", "Shaders")):
        print("reference shaders not found", file=sys.stderr)
        return 1
    print(build(a.reference, a.j))
    return 0


if __name__ == "__main__":
    sys.exit(main())
