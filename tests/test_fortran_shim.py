"""The Fortran binding module (fortran/m_tristan_gpu.F90) against the C
header: every bind(C) interface names a function include/tristan_gpu.h
declares, with the same number of arguments. No Fortran compiler exists
here, so this is what keeps the shim and the C-ABI in step."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tristan_gpu.h")
SHIM = os.path.join(ROOT, "tristan-mp-pu-master_densdecomp_gb300", "fortran", "m_tristan_gpu.F90")


def c_declarations():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"(?:int|void|const char|int32_t|int64_t|double)\s*\**\s*(tg_\w+)\s*\(([^)]*)\)\s*;", text):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = len(params)
    return out


def fortran_bindings():
    text = re.sub(r"&\s*\n\s*", " ", open(SHIM).read())
    out = {}
    for m in re.finditer(r"(?:function|subroutine)\s+\w+\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(tg_\w+)\"\)", text):
        out[m.group(2)] = len([a for a in m.group(1).split(",") if a.strip()])
    return out


def test_every_binding_matches_a_declaration():
    decl, bound = c_declarations(), fortran_bindings()
    assert len(bound) >= 40
    for name, nargs in bound.items():
        assert name in decl, name
        assert decl[name] == nargs, (name, nargs, decl[name])


def test_main_loop_calls_are_bound():
    """the calls a Fortran main loop makes per lap and around output"""
    need = {"tg_init", "tg_finalize", "tg_bind_fields", "tg_bind_particles", "tg_sync_to_host",
            "tg_sync_from_host", "tg_bc_b1", "tg_bc_e1", "tg_advance_b_half", "tg_advance_e", "tg_move",
            "tg_reset_currents", "tg_deposit", "tg_fold_currents", "tg_filter", "tg_add_current", "tg_reorder",
            "tg_step", "tg_step_host", "tg_pin_host", "tg_set_host_parts", "tg_diag_fp64", "tg_get_counts",
            "tg_output_var", "tg_output_particles", "tg_spectrum", "tg_spectrum_x", "tg_moments",
            "tg_write_restart", "tg_read_restart", "tg_last_error"}
    assert need <= set(fortran_bindings())


# the hot-path calls of the reference's lap body (code/tristanmainloop.F90:
# 117-303) that the shim replaces under the same names
LAP_CALLS = ("bc_b1", "bc_e1", "bc_b2", "bc_e2", "advance_Bhalfstep", "advance_Efield", "move_particles",
             "reset_currents", "deposit_particles", "exchange_current", "apply_filter1_opt", "add_current",
             "reorder_particles")
HOOKS = ("particle_bc_user", "field_bc_user", "inject_particles_user")


def shim_text():
    return re.sub(r"&\s*\n\s*", " ", open(SHIM).read())


def test_shim_exports_the_reference_names():
    text = shim_text()
    public = set()
    for m in re.finditer(r"public\s*::\s*([^\n]*)", text):
        public |= {a.strip() for a in m.group(1).split(",") if a.strip()}
    for name in LAP_CALLS + HOOKS:
        assert name in public, name
        assert re.search(r"\n\s*subroutine\s+%s\s*\(\s*\)" % name, text), name


def test_shim_renames_the_cpu_versions_it_imports():
    """m_fields exports advance_Efield, advance_Bhalfstep, add_current and
    reset_currents (code/fields.F90:115-116), m_particles reorder_particles
    (code/particles.F90:137): the shim's use lines rename them away so its
    own procedures can carry those names"""
    text = shim_text()
    for mod, names in (("m_fields", ("advance_Efield", "advance_Bhalfstep", "add_current", "reset_currents")),
                       ("m_particles", ("reorder_particles",))):
        for suffix in ("", "_3d"):
            line = re.search(r"\n\s*use %s%s\s*,([^\n]*)" % (mod, suffix), text)
            assert line, mod + suffix
            for n in names:
                assert re.search(r"\w+\s*=>\s*%s\b" % n, line.group(1)), (mod + suffix, n)


# ---------------------------------------------------------------------------
# bind(C) derived types against the C structs: field names, order, offsets
# and sizes under C layout rules (each member aligned to its own size, the
# struct padded to its largest member)
# ---------------------------------------------------------------------------
F_SIZES = {"c_int32_t": 4, "c_int": 4, "c_float": 4, "c_int64_t": 8, "c_double": 8}


def fortran_struct_layouts():
    text = shim_text()
    out = {}
    for m in re.finditer(r"type\s*,\s*bind\(C\)\s*::\s*(\w+)(.*?)end type", text, flags=re.S):
        fields, off, align = [], 0, 1
        for decl in m.group(2).splitlines():
            d = re.match(r"\s*(?:integer|real)\((\w+)\)\s*::\s*(.*)", decl.split("!")[0])
            if not d:
                continue
            size = F_SIZES[d.group(1)]
            for item in re.findall(r"(\w+)(?:\((\d+)\))?", d.group(2)):
                name, count = item[0], int(item[1] or 1)
                off = (off + size - 1) // size * size
                fields.append((name, off))
                off += size * count
                align = max(align, size)
        out[m.group(1)] = (fields, (off + align - 1) // align * align)
    return out


def test_bind_c_types_match_the_c_structs(tmp_path):
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        import pytest
        pytest.skip("no C compiler")
    layouts = fortran_struct_layouts()
    assert {"tg_config", "tg_shock", "tg_diag", "tg_restart_meta"} <= set(layouts)
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "tristan_gpu.h"', "int main(void) {"]
    for t, (fields, _) in layouts.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (t, t))
        for name, _ in fields:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (t, name, t, name))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)]).decode().splitlines())
    for t, (fields, size) in layouts.items():
        assert int(got[t]) == size, (t, size, got[t])
        for name, off in fields:
            assert int(got[t + "." + name]) == off, (t, name, off, got[t + "." + name])
    # every member of the C structs is in the Fortran type (same count)
    header = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    structs = {m.group(2): m.group(1) for m in re.finditer(r"typedef struct \{([^{}]*)\}\s*(\w+);", header)}
    for t, (fields, _) in layouts.items():
        cnames = re.findall(r"(\w+)(?:\[\d+\])?\s*[,;]", structs[t])
        assert [n for n, _ in fields] == cnames, t
