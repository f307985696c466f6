"""Recipe: compile the reference's own lighting-path sources on the host.

TEST INFRASTRUCTURE ONLY (oracle pinning). Reads the VoxelEngine sources where
they lie ($VXL_REFERENCE_DIR, else the tree `reference` beside this
checkout) and writes every
output into oracle/_ref/ (git-ignored):

* Sources/Shaders/lib/Light.frag is compiled as C++ against the reference's
  vendored glm (Vendor/glm). Two mechanical edits turn GLSL into C++: the
  `out vec3 x` parameter qualifier becomes `vec3& x`, and multi-component
  swizzles `.xyz` become glm's swizzle functions `.xyz()`. `texelFetch`,
  `textureSize` and SHADOW_VOX_TEXTURE are provided by ref_light_harness.cpp
  (an R8 byte grid with robust out-of-range reads and a fetch counter).
  Common.frag is skipped by predefining its include guard.
* The ray-setup blocks of LightAmbient.frag (cosineSampleHemisphere,
  calculateAmbientIrradiance, the sun-shadow setup), LightReflection.frag,
  LightPoint.frag and LightSpot.frag are cut out between anchor lines and
  compiled inside wrapper functions of the harness.
* Sources/World/Systems/ShadowVoxSystem.cpp is compiled unmodified against the
  stand-in headers in oracle/ref/shim/ (engine, Vulkan and entt types).
* clipToAABB and intersectVolume are cut out of Sources/Shaders/GeometryVoxel.frag
  (same two edits, plus `out uint` -> `uint&`) and compiled inside
  ref_geometry_harness.cpp with a three-mip R8 volume; the mip loop of
  VoxAsset::Upload (Sources/Asset/VoxAsset.cpp) is cut out and compiled there too.
* TransformSystem::RealculateMatrix (Sources/World/Systems/TransformSystem.cpp)
  is cut out, made a free function, and compiled in ref_transform_harness.cpp
  against the vendored glm; so is the picking DDA RayVoxCast
  (Sources/World/Systems/PhysicsSystem.cpp), unmodified, with stand-ins for
  the engine's asset reference and VoxAsset::PixelAt.
* main and luminance of Sources/Shaders/LightTAA.frag are cut out (main renamed
  taa_main; assignments to a .xyz swizzle rewritten component-wise) and
  compiled in ref_taa_harness.cpp with the library's bilinear sampler.

Compiler flags: -O2 -ffp-contract=off -fsingle-precision-constant (GLSL float
literals are single precision). Output: oracle/_ref/libvxl_ref.so.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SO = os.path.join(OUT, "libvxl_ref.so")


def reference_dir() -> str:
    """$VXL_REFERENCE_DIR, else a VoxelEngine tree named `reference` beside
    this checkout."""
    checkout = os.path.dirname(ORACLE)
    return os.environ.get("VXL_REFERENCE_DIR", os.path.join(os.path.dirname(checkout), "reference"))


def available() -> bool:
    r = reference_dir()
    return os.path.exists(os.path.join(r, "Sources", "Shaders", "lib", "Light.frag")) and os.path.exists(
        os.path.join(r, "Vendor", "glm", "glm.hpp")
    )


def _glslpp(text: str) -> str:
    text = re.sub(r"\bout\s+vec3\s+", "vec3& ", text)
    text = re.sub(r"\bout\s+uint\s+", "uint& ", text)
    text = re.sub(r"\.([xyzw]{2,4})\b(?!\s*\()", r".\1()", text)
    text = re.sub(r"\.([rgba]{2,4})\b(?!\s*\()", r".\1()", text)
    return text


def _swizzle_assign(text: str) -> str:
    """GLSL assignments to a .xyz swizzle (`v.xyz op= e;`) as component-wise C++."""
    def rep(m):
        v, op, e = m.group(1), m.group(2), m.group(3)
        return ("{ vec3 _t(%s.x, %s.y, %s.z); _t %s (%s); %s.x = _t.x; %s.y = _t.y; %s.z = _t.z; }"
                % (v, v, v, op, e, v, v, v))
    return re.sub(r"\b(\w+)\.xyz\s*(\+=|-=|\*=|/=|=)\s*([^;]+);", rep, text)


def _function(src: str, signature: str) -> str:
    i = src.index(signature)
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[i : k + 1]
    raise ValueError("unbalanced braces after " + signature)


def _block(src: str, start: str, end: str) -> str:
    lines = src.splitlines()
    s = next(i for i, l in enumerate(lines) if start in l)
    e = next(i for i in range(s, len(lines)) if end in lines[i])
    return "\n".join(lines[s : e + 1])


def _braced_from(src: str, start: str) -> str:
    """From the line holding `start` to the brace that closes the block it opens."""
    i = src.index(start)
    i = src.rindex("\n", 0, i) + 1
    j = src.index("{", i)
    depth = 0
    for k in range(j, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[i : k + 1]
    raise ValueError("unbalanced braces after " + start)


def generate() -> None:
    r = reference_dir()
    sh = os.path.join(r, "Sources", "Shaders")
    os.makedirs(OUT, exist_ok=True)
    light = open(os.path.join(sh, "lib", "Light.frag")).read()
    amb = open(os.path.join(sh, "LightAmbient.frag")).read()
    refl = open(os.path.join(sh, "LightReflection.frag")).read()
    point = open(os.path.join(sh, "LightPoint.frag")).read()
    spot = open(os.path.join(sh, "LightSpot.frag")).read()
    geo = open(os.path.join(sh, "GeometryVoxel.frag")).read()
    voxasset = open(os.path.join(r, "Sources", "Asset", "VoxAsset.cpp")).read()
    transform = open(os.path.join(r, "Sources", "World", "Systems", "TransformSystem.cpp")).read()
    physics = open(os.path.join(r, "Sources", "World", "Systems", "PhysicsSystem.cpp")).read()
    taa = open(os.path.join(sh, "LightTAA.frag")).read()
    parts = {
        "geometry_clip.inc": _glslpp(_function(geo, "vec3 clipToAABB(")),
        "geometry_intersect.inc": _glslpp(_function(geo, "bool intersectVolume(")),
        "voxasset_mip.inc": _braced_from(voxasset, "for (int x = 0; x < mipSizeX; x++)"),
        "taa_main.inc": _glslpp(_swizzle_assign(_function(taa, "float luminance(") + "\n"
                                                 + _function(taa, "void main()").replace("void main()",
                                                                                         "void taa_main()", 1))),
        "transform_realculate.inc": _function(transform, "void TransformSystem::RealculateMatrix(").replace(
            "TransformSystem::", "", 1),
        "physics_rayvox.inc": _function(physics, "bool RayVoxCast("),
        "Light_frag.inc": _glslpp(light),
        "ambient_cosine.inc": _glslpp(_function(amb, "vec3 cosineSampleHemisphere(")),
        "ambient_irradiance.inc": _glslpp(_function(amb, "vec3 calculateAmbientIrradiance(")),
        "ambient_sundir.inc": _glslpp(_block(amb, "const vec3 SUN_DIR", "const vec3 SUN_DIR") + "\n"
                                      + _block(amb, "const float AMBIENT_LIGHT_FACTOR", "const float AMBIENT_LIGHT_FACTOR")),
        "ambient_shadow_setup.inc": _glslpp(_block(amb, "vec3 wd = SUN_DIR;", "float bias =")),
        "reflection_cosine.inc": _glslpp(_function(refl, "vec3 cosineSampleHemisphere(")),
        "reflection_setup.inc": _glslpp(_block(refl, "vec3 wd = normalize((GetInverseViewMatrix()", "wd *= 1.0+")),
        "point_setup.inc": _glslpp(_block(point, "vec3 wd = lightDir;", "wcp += randomVec*2.5;")),
        "spot_setup.inc": _glslpp(_block(spot, "vec3 wd = normalize(lightDir)*10.0;", "wcp += randomVec*2.5;")),
    }
    # LightReflection.frag carries its own copy of cosineSampleHemisphere; the
    # harness compiles LightAmbient.frag's, so require the two to be identical.
    if parts["reflection_cosine.inc"] != parts["ambient_cosine.inc"]:
        raise RuntimeError("cosineSampleHemisphere differs between LightAmbient.frag and LightReflection.frag")
    for name, text in parts.items():
        with open(os.path.join(OUT, name), "w") as f:
            f.write("// generated by oracle/ref/build_ref.py from the reference sources; not committed\n")
            f.write(text + "\n")


def build(force: bool = False, verbose: bool = False) -> str | None:
    """Build oracle/_ref/libvxl_ref.so; returns its path, or None if the reference is absent."""
    if not available():
        return None
    srcs = [os.path.join(HERE, "ref_light_harness.cpp"), os.path.join(HERE, "ref_voxelizer_harness.cpp"),
            os.path.join(HERE, "ref_geometry_harness.cpp"), os.path.join(HERE, "ref_transform_harness.cpp"),
            os.path.join(HERE, "ref_taa_harness.cpp")]
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= max(os.path.getmtime(s) for s in srcs + [__file__]):
        return SO
    generate()
    r = reference_dir()
    common = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
              "-fsingle-precision-constant", "-w"]
    objs = []
    # Light.frag and the pass blocks
    o1 = os.path.join(OUT, "ref_light.o")
    subprocess.run(common + ["-c", "-I", OUT, "-I", os.path.join(r, "Sources", "Shaders", "lib"),
                             "-I", os.path.join(r, "Vendor"), srcs[0], "-o", o1], check=True)
    objs.append(o1)
    # ShadowVoxSystem.cpp, unmodified, against the stand-in headers
    o2 = os.path.join(OUT, "ref_shadowvox.o")
    subprocess.run(common + ["-c", "-I", os.path.join(HERE, "shim"), "-I", os.path.join(r, "Vendor"),
                             os.path.join(r, "Sources", "World", "Systems", "ShadowVoxSystem.cpp"), "-o", o2],
                   check=True)
    objs.append(o2)
    o3 = os.path.join(OUT, "ref_vox_harness.o")
    subprocess.run(common + ["-c", "-I", os.path.join(HERE, "shim"), "-I", os.path.join(r, "Vendor"),
                             "-I", os.path.join(r, "Sources", "World", "Systems"), srcs[1], "-o", o3], check=True)
    objs.append(o3)
    # GeometryVoxel.frag's clipToAABB / intersectVolume and VoxAsset::Upload's mip loop
    o4 = os.path.join(OUT, "ref_geometry.o")
    subprocess.run(common + ["-c", "-I", OUT, "-I", os.path.join(r, "Vendor"), srcs[2], "-o", o4], check=True)
    objs.append(o4)
    # TransformSystem::RealculateMatrix (no -fsingle-precision-constant needed: C++ source)
    o5 = os.path.join(OUT, "ref_transform.o")
    subprocess.run(common + ["-c", "-I", OUT, "-I", os.path.join(r, "Vendor"), srcs[3], "-o", o5], check=True)
    objs.append(o5)
    # LightTAA.frag's main and luminance
    o6 = os.path.join(OUT, "ref_taa.o")
    subprocess.run(common + ["-c", "-I", OUT, "-I", os.path.join(r, "Vendor"), srcs[4], "-o", o6], check=True)
    objs.append(o6)
    tmp = SO + ".tmp%d" % os.getpid()
    subprocess.run(["g++", "-shared", "-o", tmp] + objs, check=True)
    os.replace(tmp, SO)
    if verbose:
        print("built", SO)
    return SO


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    if p is None:
        print("reference sources not found; nothing built")
