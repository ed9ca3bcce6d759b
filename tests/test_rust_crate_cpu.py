"""The mm3e-cuda Rust crate (shipped as source; no Rust toolchain here) mirrors the C ABI.

Its `#[repr(C)]` structs must hold the header's members in the header's order with the same
types and array lengths, its constants the header's values, and its extern block the header's
entry points with their parameter counts. Parsed from both sources as text.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mm3e_cuda.h")
CRATE = os.path.join(ROOT, "atom-3d-engine_gb300", "rust", "mm3e-cuda")

C_TYPES = {"uint32_t": "u32", "float": "f32", "double": "f64", "uint64_t": "u64", "int": "c_int"}


def _strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def header_structs():
    text = _strip_c_comments(open(HEADER).read())
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", text, flags=re.S):
        fields = []
        for line in m.group(2).split(";"):
            line = line.strip()
            if not line:
                continue
            parts = line.split()
            ctype = " ".join(parts[:-1]) if "," not in line else parts[0]
            names = line[len(ctype):].split(",")
            for nm in names:
                nm = nm.strip()
                arr = re.match(r"(\*?)(\w+)(?:\[(\d+)\])?", nm)
                ptr, name, n = arr.group(1), arr.group(2), arr.group(3)
                base = ctype.replace("const ", "").strip()
                if ptr or base.endswith("*"):
                    ty = "ptr"
                else:
                    ty = C_TYPES.get(base, base)
                fields.append((name, ty, int(n) if n else None))
        out[m.group(1)] = fields
    return out


def crate_structs():
    text = open(os.path.join(CRATE, "src", "ffi.rs")).read()
    out = {}
    for m in re.finditer(r"pub struct (\w+) \{(.*?)\n\}", text, flags=re.S):
        fields = []
        for fm in re.finditer(r"pub (\w+): ([^,\n]+),", m.group(2)):
            name, ty = fm.group(1), fm.group(2).strip()
            am = re.match(r"\[(\w+); (\d+)\]", ty)
            if ty.startswith("*"):
                fields.append((name, "ptr", None))
            elif am:
                fields.append((name, am.group(1), int(am.group(2))))
            else:
                fields.append((name, ty, None))
        out[m.group(1)] = fields
    return out


def test_crate_structs_mirror_the_header_field_for_field():
    h, r = header_structs(), crate_structs()
    mirrored = ["mm3e_object", "mm3e_material", "mm3e_light", "mm3e_marcher", "mm3e_post", "mm3e_csg_node",
                "mm3e_volume", "mm3e_gi", "mm3e_scene_desc", "mm3e_camera", "mm3e_dyn_sphere", "mm3e_render_stats"]
    for name in mirrored:
        assert name in h and name in r, name
        hf = [(n, "ptr" if t == "ptr" else t, k) for n, t, k in h[name]]
        rf = r[name]
        # the header's nested struct members keep their type names
        hf = [(n, t if t in ("u32", "f32", "f64", "u64", "ptr") else t, k) for n, t, k in hf]
        assert [f[0] for f in hf] == [f[0] for f in rf], (name, hf, rf)
        for (hn, ht, hk), (rn, rt, rk) in zip(hf, rf):
            assert hk == rk, (name, hn, hk, rk)
            if ht in ("mm3e_marcher", "mm3e_post"):
                assert rt == ht, (name, hn, rt)
            else:
                assert ht == rt, (name, hn, ht, rt)


def test_crate_constants_match_the_header():
    text = _strip_c_comments(open(HEADER).read())
    hvals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(MM3E_\w+)\s*=\s*(-?\d+)", text)}
    hvals.update({m.group(1): int(m.group(2)) for m in re.finditer(r"#define (MM3E_ABI_VERSION) (\d+)", text)})
    rs = open(os.path.join(CRATE, "src", "ffi.rs")).read()
    consts = re.findall(r"pub const (MM3E_\w+): \w+ = (-?\d+);", rs)
    assert len(consts) >= 35
    for name, val in consts:
        assert name in hvals, name
        assert hvals[name] == int(val), name


def test_crate_entry_points_exist_with_their_arity():
    text = _strip_c_comments(open(HEADER).read())
    harity = {}
    for m in re.finditer(r"\b(?:int|void|const char\*)\s+(mm3e_\w+)\s*\(([^;]*?)\);", text, flags=re.S):
        args = m.group(2).strip()
        harity[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    rs = open(os.path.join(CRATE, "src", "ffi.rs")).read()
    block = rs[rs.index('extern "C" {'):]
    fns = re.findall(r"pub fn (mm3e_\w+)\((.*?)\)", block, flags=re.S)
    assert len(fns) >= 10
    for name, args in fns:
        assert name in harity, name
        n = 0 if not args.strip() else len([a for a in args.split(",") if a.strip()])
        assert n == harity[name], (name, n, harity[name])


def test_crate_files_present():
    for f in ("Cargo.toml", "build.rs", os.path.join("src", "lib.rs"), os.path.join("src", "ffi.rs")):
        assert os.path.exists(os.path.join(CRATE, f)), f
    lib = open(os.path.join(CRATE, "src", "lib.rs")).read()
    for api in ("pub fn compile(&self, scene: Arc<Scene>) -> Result<CudaScene, String>",
                "pub fn try_render(&self, camera: &Camera, dyn_spheres: &[DynSphere]) -> Result<Framebuffer, String>",
                "pub fn render_linear(&self, camera: &Camera) -> Result<Vec<Vec3>, String>",
                "pub fn bake_gi(&self, dims: (u32, u32, u32), samples: u32) -> Result<(), String>"):
        assert api in lib, api
