"""The C-ABI library loads and exports every entry point include/*.h declares;
the mixture structs of include/htr_mix.h are byte-compatible with the
reference's `struct Mix`; the CPU oracle exports the same task entry points.
No compute call is made here (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from htr_gb300 import abi, runtime

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|size_t|char\s*\*|const char\s*\*|void)\s*\**\s*(htr_\w+)\s*\(", re.M)


def declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            with open(os.path.join(ROOT, "include", h)) as f:
                names |= set(DECL.findall(f.read()))
    return sorted(names)


def test_headers_declare_the_task_set():
    names = declared()
    for d in "XYZ":
        for s in ("Hybrid", "TENO", "TENOA", "TENOLAD", "SkewSymmetric"):
            assert f"htr_UpdateUsing{s}EulerFlux{d}" in names
        assert f"htr_UpdateUsingDiffusionFlux{d}" in names
        assert f"htr_UpdateShockSensor{d}" in names
    for n in ("htr_UpdateDucrosSensor", "htr_AddChemistrySources", "htr_UpdateChemistry",
              "htr_load_mixture", "htr_rk3_step", "htr_rk3_step_ws", "htr_rk3_workspace_bytes"):
        assert n in names


def test_library_exports_every_declared_symbol():
    if not os.path.exists(runtime.LIB_PATH):
        pytest.skip("CUDA library not built")
    lib = C.CDLL(runtime.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_oracle_exports_the_task_entry_points():
    port = oracle.port_lib()
    tasks = [n for n in declared() if n.startswith(("htr_UpdateUsing", "htr_UpdateShock", "htr_UpdateDucros",
                                                    "htr_AddChemistry", "htr_UpdateChemistry",
                                                    "htr_Update", "htr_Calculate", "htr_Initialize"))]
    missing = [n for n in tasks if not hasattr(port, n)]
    assert not missing, missing


@pytest.mark.parametrize("eos", [abi.HTR_EOS_CONSTPROPMIX, abi.HTR_EOS_AIRMIX])
def test_mixture_struct_layout_matches_reference(eos):
    ref = oracle.ref_lib(eos)
    if ref is None:
        pytest.skip("reference CPU build not present on this machine")
    S = abi.MIX_STRUCT[eos]
    assert C.sizeof(S) == ref.htr_ref_mix_sizeof()
    buf = (C.c_longlong * 16)()
    n = ref.htr_ref_mix_offsets(buf, 16)
    if eos == abi.HTR_EOS_CONSTPROPMIX:
        mine = [S.R.offset, S.gamma.offset, S.viscosityModel.offset, S.constantVisc.offset,
                S.powerlawViscRef.offset, S.Prandtl.offset]
    else:
        sp, nasa, lj = abi.htr_species_t, abi.htr_nasa9_t, abi.htr_ljdata_t
        rx, tb = abi.htr_reaction_t, abi.htr_tbreaction_t
        mine = [C.sizeof(sp), sp.W.offset, sp.cpCoeff.offset + nasa.cpL.offset,
                sp.DiffCoeff.offset + lj.Z298.offset, S.reactions.offset,
                S.reactions.offset + C.sizeof(rx) + rx.pducts.offset + C.sizeof(abi.htr_stoich_t)
                + abi.htr_stoich_t.nu.offset,
                S.ThirdbodyReactions.offset,
                S.ThirdbodyReactions.offset + 2 * C.sizeof(tb) + tb.thirdb.offset + 4 * C.sizeof(abi.htr_collider_t)
                + abi.htr_collider_t.eff.offset,
                S.PRef.offset, S.TMin.offset]
    assert list(buf[:n]) == mine


def test_product_mixture_builder_matches_reference():
    ref = oracle.ref_lib(abi.HTR_EOS_AIRMIX)
    if ref is None or not os.path.exists(runtime.LIB_PATH):
        pytest.skip("needs the reference CPU build and the CUDA library")
    from tests import util
    lib = C.CDLL(runtime.LIB_PATH)
    abi.bind(lib)
    xi = (C.c_double * 5)(0.79, 0.21, 0.0, 0.0, 0.0)
    a, b = abi.htr_airmix_t(), abi.htr_airmix_t()
    assert lib.htr_airmix_init(101325.0, 300.0, 1.0, xi, C.byref(a)) == 0
    assert ref.htr_airmix_init(101325.0, 300.0, 1.0, xi, C.byref(b)) == 0
    assert not util.struct_diff(a, b)
