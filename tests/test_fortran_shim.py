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
