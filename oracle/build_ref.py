"""Build the reference-side parity checkers into oracle/_ref/ (TEST INFRASTRUCTURE).

Everything here is compiled from the reference's own sources where they lie
(a read-only checkout of tkhenry-uofa/ogl_beamforming_cuda); nothing of the
reference is copied into the repository. Outputs go to oracle/_ref/ only, which
is git-ignored.

  libref_math.so    the reference's math.c (make_hadamard_transpose,
                    kaiser_low_pass_filter, matched_filter, cephes I0) and
                    das_voxel_transform_matrix (beamformer.c:483-518, cut out of
                    beamformer.c by function name), behind ref_math_wrap.c.
  libref_client.so  helpers/ogl_beamformer_lib.c unchanged: the reference client
                    library, for ABI and error-path comparisons (it has no server
                    here, so every call that needs one fails with SHARED_MEMORY).
  libref_shaders.so the compute shaders decode/filter/das/sum/min_max.glsl
                    compiled as C++20 through glsl_shim.hpp. Only the resource
                    declarations (`layout(...) buffer/uniform` lines) are
                    rewritten into C++ declarations; function bodies compile as
                    written. ref_shader_driver.cpp runs their dispatch grids.
  zemp_probe        the zemp_bp_v1 typedef of tests/throughput.c (the captured-
                    dataset parameter block), cut out by name and compiled into
                    a program printing its size and field offsets.
  parameters_layout.txt  field offsets of BeamformerParameters and the sizes of
                    its sibling structs, printed by a probe that includes the
                    reference's beamformer_parameters.h.

Usage: python oracle/build_ref.py --reference PATH (or BF_REFERENCE_DIR=PATH).
Exits 0 and builds nothing when no checkout is given or it is absent.
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# decode.glsl variants: (namespace, defines) -- shader_text_with_header, beamformer.c:762-783
DECODE_VARIANTS = [
    ("decode_i16", []),
    ("decode_i16c", ["INPUT_DATA_TYPE_INT16_COMPLEX"]),
    ("decode_f32", ["INPUT_DATA_TYPE_FLOAT"]),
    ("decode_f32c", ["INPUT_DATA_TYPE_FLOAT_COMPLEX"]),
    ("decode_i16_to_f32", ["OUTPUT_DATA_TYPE_FLOAT"]),
]
# filter.glsl variants -- beamformer.c:718-733
FILTER_VARIANTS = [
    ("filter_f32c", ["INPUT_DATA_TYPE_FLOAT"]),
    ("demod_i16", ["DEMODULATE"]),
    ("demod_f32", ["INPUT_DATA_TYPE_FLOAT", "DEMODULATE"]),
]
DAS_VARIANTS = [("das_full", ["DAS_FAST 0"]), ("das_fast", ["DAS_FAST 1"])]
PARAMETER_FIELDS = ("xdc_transform", "dec_data_dim", "xdc_element_pitch", "rf_raw_dim", "transmit_mode", "decode",
                    "das_shader_id", "time_offset", "output_min_coordinate", "output_max_coordinate", "output_points",
                    "sampling_frequency", "center_frequency", "speed_of_sound", "off_axis_pos", "beamform_plane",
                    "f_number", "interpolate", "coherency_weighting", "decimation_rate", "readi_group_id",
                    "readi_group_size")

DECODE_UBO = """
static uint input_channel_stride, input_sample_stride, input_transmit_stride;
static uint output_channel_stride, output_sample_stride, output_transmit_stride;
static uint transmit_count, decode_mode;
static bool u_first_pass;
#define DECODE_MODE_NONE 0
#define DECODE_MODE_HADAMARD 1
"""
FILTER_UBO = """
static uint input_channel_stride, input_sample_stride, input_transmit_stride;
static uint output_channel_stride, output_sample_stride, output_transmit_stride;
static uint decimation_rate;
static bool map_channels;
static float demodulation_frequency, sampling_frequency;
"""
# The DAS uniform block is produced from the reference's own X-macro lists, the
# same way static.c:411-431 builds the GLSL header text.
DAS_UBO = """
#define X(name, type, size, __e, gltype, glsize, comment) static gltype name glsize;
BEAMFORMER_PARAMS_HEAD
BEAMFORMER_UI_PARAMS
BEAMFORMER_PARAMS_TAIL
#undef X
static ivec3 u_voxel_offset;
static mat4  u_voxel_transform;
static uint  u_cycle_t;
static int   u_channel;
#define X(type, id, pretty, fixed_tx) enum { DAS_ID_##type = id };
DAS_TYPES
#undef X
"""
SUM_UBO = "static float u_sum_prescale = 1.0f;\n"
MINMAX_UBO = "static int u_mip_map;\n"


def translate(src):
    """Rewrite GLSL resource declarations into C++ declarations."""
    src = re.sub(r"layout\s*\(\s*local_size[^)]*\)\s*in\s*;", "", src)
    src = re.sub(
        r"layout\s*\([^)]*\)\s*(?:(?:readonly|writeonly|restrict)\s+)*buffer\s+\w+\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;",
        r"static glsl::ssbo<\1> \2;", src)
    src = re.sub(
        r"layout\s*\([^)]*\)\s*(?:(?:readonly|writeonly|restrict)\s+)*uniform\s+(\w+)\s+(\w+)\s*;",
        r"static \1 \2;", src)
    src = src.replace("gl_GlobalInvocationID.xyz", "gl_GlobalInvocationID")
    return src


def defined_macros(src):
    return sorted(set(re.findall(r"^\s*#\s*define\s+(\w+)", src, re.M)))


def emit(ns, header, defines, body):
    out = [f"namespace glsl {{ namespace {ns} {{"]
    for d in defines:
        name, _, val = d.partition(" ")
        out.append(f"#define {name} {val}".rstrip())
    out.append("#define main shader_main")
    out.append(header)
    out.append(body)
    out.append("#undef main")
    for d in defines:
        out.append(f"#undef {d.partition(' ')[0]}")
    for m in defined_macros(body):
        out.append(f"#undef {m}")
    out.append("}}")
    return "\n".join(out) + "\n"


def extract_function(text, name):
    """Cut `function <type>\\nname(...) { ... }` out of a C file by brace matching."""
    m = re.search(r"function\s+\w+\s*\n" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise RuntimeError(f"{name} not found")
    i = text.index("{", m.end())
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[m.start():j + 1]
    raise RuntimeError(f"{name}: unbalanced braces")


def run(cmd):
    print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)


def build(ref):
    os.makedirs(OUT, exist_ok=True)
    shaders = os.path.join(ref, "shaders")
    parts = ['#include "glsl_shim.hpp"\n', '#include "beamformer_parameters.h"\n']
    dec = translate(open(os.path.join(shaders, "decode.glsl")).read())
    for ns, defs in DECODE_VARIANTS:
        parts.append(emit(ns, DECODE_UBO, defs, dec))
    flt = translate(open(os.path.join(shaders, "filter.glsl")).read())
    for ns, defs in FILTER_VARIANTS:
        parts.append(emit(ns, FILTER_UBO, defs, flt))
    das = translate(open(os.path.join(shaders, "das.glsl")).read())
    for ns, defs in DAS_VARIANTS:
        parts.append(emit(ns, DAS_UBO, defs, das))
    parts.append(emit("sum", SUM_UBO, [], translate(open(os.path.join(shaders, "sum.glsl")).read())))
    parts.append(emit("min_max", MINMAX_UBO, [], translate(open(os.path.join(shaders, "min_max.glsl")).read())))
    gen = os.path.join(OUT, "ref_shaders_gen.inc")
    with open(gen, "w") as f:
        f.write("/* generated by oracle/build_ref.py from the reference's shaders; do not commit */\n")
        f.write("".join(parts))

    bf = open(os.path.join(ref, "beamformer.c")).read()
    with open(os.path.join(OUT, "ref_voxel_gen.inc"), "w") as f:
        f.write("/* generated by oracle/build_ref.py; do not commit */\n")
        f.write(extract_function(bf, "das_voxel_transform_matrix") + "\n")

    cxx = ["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-strict-aliasing", "-w", f"-I{HERE}", f"-I{OUT}", f"-I{ref}"]
    run(cxx + [os.path.join(HERE, "ref_shader_driver.cpp"), "-o", os.path.join(OUT, "libref_shaders.so")])
    # the reference's own optimisation flags (build.c:31-35), without -march=native
    cc = ["gcc", "-std=c11", "-O3", "-funsafe-math-optimizations", "-fno-math-errno", "-fPIC", "-shared", "-w",
          f"-I{ref}", f"-I{OUT}"]
    run(cc + [os.path.join(HERE, "ref_math_wrap.c"), "-o", os.path.join(OUT, "libref_math.so"), "-lm"])
    # layout of the reference's dataset header (zemp_bp_v1, tests/throughput.c): the
    # typedef is cut from the file and compiled into a probe printing size and offsets
    tp = open(os.path.join(ref, "tests", "throughput.c")).read()
    m = re.search(r"#define ZEMP_BP_MAGIC.*?\n(typedef struct \{.*?\} zemp_bp_v1;)", tp, re.S)
    if m:
        fields = re.findall(r"^\s*\w+\s+(\w+)(?:\[\d+\])?;", m.group(1), re.M)
        probe = os.path.join(OUT, "zemp_probe.c")
        with open(probe, "w") as f:
            f.write("/* generated by oracle/build_ref.py from the reference's tests/throughput.c; do not commit */\n"
                    "#include <stdint.h>\n#include <stdio.h>\n#include <stddef.h>\n"
                    "typedef uint64_t u64; typedef uint32_t u32; typedef uint16_t u16; typedef int16_t i16;\n"
                    "typedef int32_t i32; typedef float f32;\n" + m.group(1) + "\n"
                    "int main(void) {\n\tprintf(\"sizeof %zu\\n\", sizeof(zemp_bp_v1));\n" +
                    "".join(f"\tprintf(\"{n} %zu\\n\", offsetof(zemp_bp_v1, {n}));\n" for n in fields) +
                    "\treturn 0;\n}\n")
        run(["gcc", "-std=c11", probe, "-o", os.path.join(OUT, "zemp_probe")])
    run(cc + [os.path.join(ref, "helpers", "ogl_beamformer_lib.c"), "-o", os.path.join(OUT, "libref_client.so"),
              "-lm"])
    # layout of the reference's BeamformerParameters family (beamformer_parameters.h):
    # a probe that includes the header where it lies prints field offsets and sizes
    probe = os.path.join(OUT, "parameters_probe.c")
    with open(probe, "w") as f:
        f.write("#include <stdio.h>\n#include <stddef.h>\n#include <stdint.h>\n"
                f'#include "{os.path.join(ref, "beamformer_parameters.h")}"\n'
                "#define O(f) printf(#f \" %zu\\n\", offsetof(BeamformerParameters, f));\n"
                "int main(void) {\n" + "".join(f"\tO({n})\n" for n in PARAMETER_FIELDS) +
                "\tprintf(\"size %zu %zu %zu %zu %zu\\n\", sizeof(BeamformerParameters), "
                "sizeof(BeamformerUIParameters), sizeof(BeamformerParametersHead), "
                "sizeof(BeamformerComputeStatsTable), sizeof(BeamformerLiveImagingParameters));\n"
                "\treturn 0;\n}\n")
    run(["gcc", "-std=c11", probe, "-o", os.path.join(OUT, "parameters_probe")])
    layout = subprocess.run([os.path.join(OUT, "parameters_probe")], check=True, capture_output=True, text=True).stdout
    with open(os.path.join(OUT, "parameters_layout.txt"), "w") as f:
        f.write(layout)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("BF_REFERENCE_DIR"),
                    help="path of the reference checkout (default: $BF_REFERENCE_DIR)")
    args = ap.parse_args()
    if not args.reference:
        print("no reference checkout given (--reference or BF_REFERENCE_DIR); oracle/_ref not built")
        return 0
    if not os.path.isdir(os.path.join(args.reference, "shaders")):
        print(f"reference checkout not found at {args.reference}; oracle/_ref not built")
        return 0
    build(args.reference)
    return 0


if __name__ == "__main__":
    sys.exit(main())
