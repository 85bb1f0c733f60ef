"""Recipe: compile the reference's own ``.hook`` shader text as C++.

Test infrastructure.  For each ``.hook`` file of the reference named on the
command line -- root fragment-shader files, or ``compute/<name>`` for the
compute-shader form (the only form of ravu-3x) -- read in place, never copied
into the repository, this script

1. splits the file into pass blocks and texture blocks,
2. rewrites the two GLSL swizzles C++ cannot express as members
   (``.xyz`` -> ``.xyz()``, ``.wzyx`` -> ``.wzyx()``) and wraps each pass
   body in its own namespace with texture bindings from ``glsl_shim.hpp``,
3. writes the generated C++ and the texture payloads under ``oracle/_ref/``,
4. compiles one shared library per file (``g++ -O1 -ffp-contract=off``,
   evaluation in double precision) exposing

       int ref_run(const double* in, int C, int H, int W, int OW, int OH,
                   double* out, int out_cap, int* out_dims);

   which runs every enabled pass of the file in order, exactly like the mpv
   hook host would (clamp-to-edge textures, per-pixel ``hook()`` calls,
   ``//!SAVE`` / hooked-texture replacement, ``//!WIDTH``/``//!HEIGHT``/
   ``//!WHEN`` evaluated as RPN).  A ``//!COMPUTE bw bh tw th`` pass is
   dispatched over ceil(W / bw) x ceil(H / bh) workgroups of tw x th
   invocations; each workgroup runs its invocations serially in phases
   split at ``barrier()`` (``glsl_shim.hpp``, ``Compute``), ``shared``
   arrays are static, ``imageStore`` writes the pass's output texture.

The library of ``compute/<name>.hook`` is ``oracle/_ref/compute.<name>.so``.

Outputs go only to ``oracle/_ref/`` (git-ignored).  Usage::

    python oracle/build_ref.py [--ref /root/reference] [names...]
    python oracle/build_ref.py --generated [names...]

``--generated`` compiles the C++ this recipe already wrote into
``oracle/_ref/`` (for a machine of another architecture that received the
generated sources but not the reference checkout); nothing is regenerated.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = "/root/reference"

COMPUTE_DECLS = r"""
static Compute C;
#define gl_WorkGroupID (C.wg_id)
#define gl_LocalInvocationID (C.local_id)
#define gl_GlobalInvocationID (C.global_id)
#define gl_WorkGroupSize (C.wg_size)
#define gl_LocalInvocationIndex (C.local_index)
#define barrier() do { if (++C.bar > C.phase) return; } while (0)
#define shared static
static const int out_image = 0;
inline void imageStore(int, const ivec2& p, const vec4& v) { C.store(p.x, p.y, v); }
// output pixel id -> normalised input position, texel centres aligned
inline vec2 HOOKED_map(const ivec2& id) { return vec2((id.x + 0.5) / C.out->w, (id.y + 0.5) / C.out->h); }
"""
COMPUTE_MACROS = ["gl_WorkGroupID", "gl_LocalInvocationID", "gl_GlobalInvocationID", "gl_WorkGroupSize",
                  "gl_LocalInvocationIndex", "barrier", "shared"]


def out_stem(stem: str) -> str:
    """File stem under oracle/_ref of a reference path stem ("compute/x" -> "compute.x")."""
    return stem.replace("/", ".")


RPN_CPP = r"""
#include "glsl_shim.hpp"
#include <cstdlib>
#include <sstream>
#include <stdexcept>
namespace glsl {
double rpn(const char* expr, const std::map<std::string, double>& env) {
  std::vector<double> st;
  std::istringstream in(expr);
  std::string tok;
  while (in >> tok) {
    if (tok == "+" || tok == "-" || tok == "*" || tok == "/" || tok == "<" || tok == ">" || tok == "=") {
      double b = st.back(); st.pop_back();
      double a = st.back(); st.pop_back();
      double r = tok == "+" ? a + b : tok == "-" ? a - b : tok == "*" ? a * b : tok == "/" ? a / b
               : tok == "<" ? (a < b) : tok == ">" ? (a > b) : (a == b);
      st.push_back(r);
    } else if (tok == "!") {
      double a = st.back(); st.pop_back();
      st.push_back(a == 0.0 ? 1.0 : 0.0);
    } else if ((tok[0] >= '0' && tok[0] <= '9') || tok[0] == '.' || tok[0] == '-') {
      st.push_back(std::strtod(tok.c_str(), nullptr));
    } else {
      auto it = env.find(tok);
      if (it == env.end()) throw std::runtime_error("rpn: unknown " + tok);
      st.push_back(it->second);
    }
  }
  return st.back();
}
}  // namespace glsl
"""


def split_blocks(text: str):
    passes, textures = [], []
    cur = None
    lines = text.split("\n")
    i = 0
    while i < len(lines):
        ln = lines[i]
        if ln.startswith("//!DESC"):
            cur = {"dirs": {"BIND": []}, "body": []}
            passes.append(cur)
        elif ln.startswith("//!TEXTURE"):
            tex = {"name": ln.split(None, 1)[1].strip(), "filter": "NEAREST"}
            i += 1
            while lines[i].startswith("//!"):
                k, v = re.match(r"//!(\w+)\s*(.*)", lines[i]).groups()
                if k == "SIZE":
                    tex["w"], tex["h"] = (int(t) for t in v.split())
                elif k == "FILTER":
                    tex["filter"] = v.strip()
                i += 1
            tex["hex"] = lines[i].strip()
            textures.append(tex)
            cur = None
        elif ln.startswith("//!") and cur is not None:
            k, v = re.match(r"//!(\w+)\s*(.*)", ln).groups()
            if k == "BIND":
                cur["dirs"]["BIND"].append(v.strip())
            else:
                cur["dirs"][k] = v.strip()
        elif cur is not None:
            cur["body"].append(ln)
        i += 1
    return passes, textures


def gen_cpp(stem: str, passes, textures) -> str:
    tex_names = {t["name"] for t in textures}
    o = ['#include "glsl_shim.hpp"', "#include <cstdio>", "#include <cstdlib>", "#include <fstream>",
         "using namespace glsl;", "static std::map<std::string, Tex> g_tex;"]
    o.append("#define float double")
    for k, p in enumerate(passes):
        body = "\n".join(p["body"])
        body = re.sub(r"\.(wzyx|xyz)\b(?!\()", r".\1()", body)
        macros = re.findall(r"^\s*#define\s+(\w+)", body, flags=re.M)
        o.append(f"namespace p{k} {{")
        o.append("static Frag F;")
        o.append("using glsl::mix; using glsl::clamp; using glsl::max; using glsl::min; using glsl::floor;"
                 " using glsl::fract; using glsl::mod; using glsl::atan; using glsl::sqrt; using glsl::inversesqrt;"
                 " using glsl::log2; using glsl::exp; using glsl::abs; using glsl::dot; using glsl::matrixCompMult;"
                 " using glsl::outerProduct;")
        o.append("#define HOOKED_pos (F.pos)")
        o.append("#define HOOKED_size (F.size)")
        o.append("#define HOOKED_pt (vec2(1.0 / F.size.x, 1.0 / F.size.y))")
        o.append("inline vec4 texture(const Tex* t, const vec2& uv) { return t->sample(uv); }")
        compute = "COMPUTE" in p["dirs"]
        if compute:
            o.append(COMPUTE_DECLS)
        for b in p["dirs"]["BIND"]:
            if b in tex_names:
                o.append(f"static const Tex* {b} = nullptr;")
            else:
                o.append(f"static const Tex* t_{b} = nullptr;")
                o.append(f"inline vec4 {b}_texOff(const vec2& off) {{ return tex_off(*t_{b}, F, off); }}")
                o.append(f"inline vec4 {b}_tex(const vec2& uv) {{ return t_{b}->sample(uv); }}")
                if b != "HOOKED":
                    o.append(f"#define {b}_pt (vec2(1.0 / t_{b}->w, 1.0 / t_{b}->h))")
                    o.append(f"#define {b}_size (vec2(t_{b}->w, t_{b}->h))")
                    macros = macros + [f"{b}_pt", f"{b}_size"]
        o.append(body)
        for m in macros + ["HOOKED_pos", "HOOKED_size", "HOOKED_pt"] + (COMPUTE_MACROS if compute else []):
            o.append(f"#undef {m}")
        o.append(f"}}  // namespace p{k}")
    o.append("#undef float")
    # texture loading
    o.append("static int hexv(char c) { return c <= '9' ? c - '0' : (c | 32) - 'a' + 10; }")
    o.append("static void load_lut(const char* name, const char* file, int w, int h, bool linear) {")
    o.append("  std::ifstream f(file); std::string s; std::getline(f, s);")
    o.append("  Tex t; t.w = w; t.h = h; t.linear = linear; t.px.resize((size_t)w * h);")
    o.append("  for (size_t i = 0; i < (size_t)w * h * 4; i++) {")
    o.append("    uint32_t u = 0; for (int b = 0; b < 4; b++) { u |= (uint32_t)(hexv(s[8 * i + 2 * b]) * 16 + hexv(s[8 * i + 2 * b + 1])) << (8 * b); }")
    o.append("    float v; std::memcpy(&v, &u, 4); t.px[i / 4][(int)(i % 4)] = v; }")
    o.append("  g_tex[name] = t; }")
    o.append('extern "C" int ref_run(const double* in, int C, int H, int W, int OW, int OH, double* out, int out_cap, int* out_dims) {')
    o.append("  static bool loaded = false;")
    o.append("  if (!loaded) {")
    for t in textures:
        fn = os.path.join(OUT, f"{out_stem(stem)}__{t['name']}.hex")
        o.append(f'    load_lut("{t["name"]}", "{fn}", {t["w"]}, {t["h"]}, {"true" if t["filter"] == "LINEAR" else "false"});')
    o.append("    loaded = true; }")
    o.append("  Tex hooked; hooked.w = W; hooked.h = H; hooked.px.resize((size_t)W * H);")
    o.append("  for (int c = 0; c < C; c++) for (int y = 0; y < H; y++) for (int x = 0; x < W; x++) hooked.px[(size_t)y * W + x][c] = in[((size_t)c * H + y) * W + x];")
    o.append("  std::map<std::string, Tex> saved;")
    for k, p in enumerate(passes):
        d = p["dirs"]
        o.append("  {")
        o.append('    std::map<std::string, double> env{{"HOOKED.w", (double)hooked.w}, {"HOOKED.h", (double)hooked.h}, {"OUTPUT.w", (double)OW}, {"OUTPUT.h", (double)OH}, {"LUMA.w", (double)W}, {"LUMA.h", (double)H}};')
        when = d.get("WHEN")
        cond = f'rpn("{when}", env) != 0.0' if when else "true"
        o.append(f"    if ({cond}) {{")
        o.append("      (void)env;")
        wexpr = f'(int)rpn("{d["WIDTH"]}", env)' if "WIDTH" in d else "hooked.w"
        hexpr = f'(int)rpn("{d["HEIGHT"]}", env)' if "HEIGHT" in d else "hooked.h"
        o.append(f"      int ow = {wexpr}, oh = {hexpr};")
        o.append("      Tex res; res.w = ow; res.h = oh; res.px.resize((size_t)ow * oh);")
        for b in d["BIND"]:
            if b == "HOOKED":
                o.append(f"      p{k}::t_HOOKED = &hooked;")
            elif b in tex_names:
                o.append(f'      p{k}::{b} = &g_tex["{b}"];')
            else:
                o.append(f'      p{k}::t_{b} = &saved["{b}"];')
        o.append(f"      p{k}::F.size = vec2(hooked.w, hooked.h);")
        if "COMPUTE" in d:
            cw = [int(v) for v in d["COMPUTE"].split()]
            bw, bh = cw[0], cw[1]
            tw, th = (cw[2], cw[3]) if len(cw) >= 4 else (bw, bh)
            nbar = len(re.findall(r"\bbarrier\s*\(\s*\)", "\n".join(p["body"])))
            o.append(f"      p{k}::C.out = &res;")
            o.append(f"      p{k}::C.wg_size.x = {tw}; p{k}::C.wg_size.y = {th}; p{k}::C.wg_size.z = 1;")
            o.append(f"      for (int wy = 0; wy < (oh + {bh - 1}) / {bh}; wy++) for (int wx = 0; wx < (ow + {bw - 1}) / {bw}; wx++)")
            o.append(f"        for (int ph = 0; ph <= {nbar}; ph++) for (int ly = 0; ly < {th}; ly++) for (int lx = 0; lx < {tw}; lx++) {{")
            o.append(f"          Compute& c = p{k}::C;")
            o.append("          c.wg_id.x = wx; c.wg_id.y = wy; c.local_id.x = lx; c.local_id.y = ly;")
            o.append(f"          c.global_id.x = wx * {tw} + lx; c.global_id.y = wy * {th} + ly;")
            o.append(f"          c.local_index = ly * {tw} + lx; c.bar = 0; c.phase = ph;")
            o.append(f"          p{k}::hook();")
            o.append("        }")
        else:
            o.append("      for (int y = 0; y < oh; y++) for (int x = 0; x < ow; x++) {")
            o.append(f"        p{k}::F.pos = vec2((x + 0.5) / ow, (y + 0.5) / oh);")
            o.append(f"        res.px[(size_t)y * ow + x] = p{k}::hook();")
            o.append("      }")
        if d.get("SAVE"):
            o.append(f'      saved["{d["SAVE"]}"] = res;')
        else:
            o.append("      hooked = res;")
        o.append("    }")
        o.append("  }")
    o.append("  out_dims[0] = hooked.h; out_dims[1] = hooked.w;")
    o.append("  if ((size_t)C * hooked.w * hooked.h > (size_t)out_cap) return -1;")
    o.append("  for (int c = 0; c < C; c++) for (int y = 0; y < hooked.h; y++) for (int x = 0; x < hooked.w; x++) out[((size_t)c * hooked.h + y) * hooked.w + x] = hooked.px[(size_t)y * hooked.w + x][c];")
    o.append("  return 0;")
    o.append("}")
    return "\n".join(o) + "\n"


def build_one(ref: str, stem: str) -> str:
    src = os.path.join(ref, stem + ".hook")
    with open(src) as f:
        text = f.read()
    passes, textures = split_blocks(text)
    for t in textures:
        with open(os.path.join(OUT, f"{out_stem(stem)}__{t['name']}.hex"), "w") as f:
            f.write(t["hex"])
    cpp = os.path.join(OUT, out_stem(stem) + ".cpp")
    with open(cpp, "w") as f:
        f.write(gen_cpp(stem, passes, textures))
    so = os.path.join(OUT, out_stem(stem) + ".so")
    cmd = ["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-w",
           f"-I{HERE}", "-o", so, cpp, os.path.join(OUT, "rpn.o")]
    subprocess.run(cmd, check=True)
    return so


def compile_generated(names) -> list:
    """Compile generated ``oracle/_ref/<name>.cpp`` files (and ``rpn.cpp``)
    whose shared library is missing or older than the source."""
    def loads(so):  # a library built for another machine does not load here
        import ctypes
        try:
            ctypes.CDLL(so)
            return True
        except OSError:
            return False

    def stale(src, dst):
        return not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src)
    rpn_cpp, rpn_o = os.path.join(OUT, "rpn.cpp"), os.path.join(OUT, "rpn.o")
    if not os.path.exists(rpn_cpp):
        return []
    todo = []
    for stem in names:
        cpp, so = os.path.join(OUT, out_stem(stem) + ".cpp"), os.path.join(OUT, out_stem(stem) + ".so")
        if os.path.exists(cpp) and (stale(cpp, so) or not loads(so)):
            todo.append((cpp, so))
    if not todo:
        return []
    # rpn.o is rebuilt with them: an object carried over from another
    # machine cannot be told apart by its timestamp
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-c", f"-I{HERE}", "-o", rpn_o, rpn_cpp], check=True)

    def one(job):
        cpp, so = job
        subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fPIC", "-shared", "-w",
                        f"-I{HERE}", "-o", so, cpp, rpn_o], check=True)
        return so
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(one, todo))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("--generated", action="store_true",
                    help="compile the C++ already generated under oracle/_ref (no reference needed)")
    ap.add_argument("names", nargs="*")
    a = ap.parse_args(argv)
    if a.generated:
        names = a.names or sorted(fn[:-4] for fn in os.listdir(OUT) if fn.endswith(".cpp") and fn != "rpn.cpp") \
            if os.path.isdir(OUT) else []
        for so in compile_generated(names):
            print("built", os.path.relpath(so, HERE))
        return 0
    if not os.path.isdir(a.ref):
        print(f"reference not present at {a.ref}; nothing to build")
        return 0
    os.makedirs(OUT, exist_ok=True)
    rpn_cpp = os.path.join(OUT, "rpn.cpp")
    with open(rpn_cpp, "w") as f:
        f.write(RPN_CPP)
    subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-c", f"-I{HERE}", "-o",
                    os.path.join(OUT, "rpn.o"), rpn_cpp], check=True)
    names = a.names or sorted(fn[:-5] for fn in os.listdir(a.ref) if fn.endswith(".hook"))
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for so in ex.map(lambda s: build_one(a.ref, s), names):
            print("built", os.path.relpath(so, HERE))
    return 0


if __name__ == "__main__":
    sys.exit(main())
