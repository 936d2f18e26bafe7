"""The C-ABI library loads and exports every function include/tb.h declares
(no compute call: no GPU needed)."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "tb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tb_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(native):
    lib = native.engine_lib()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(native.ENGINE_SIGNATURES), set(names) ^ set(native.ENGINE_SIGNATURES)


def test_version_and_options(native):
    import ctypes

    lib = native.engine_lib()
    assert b"sm_103a" in lib.tb_version()
    o = native.TbOptions()
    lib.tb_options_default(ctypes.byref(o))
    assert o.dtype == native.TB_DTYPE_F32 and o.use_graphs == 1 and o.timeout_ms > 0


def test_struct_sizes_match_header(native):
    import ctypes

    # tb_options: 2 int32, int64, 3 int32, 9 reserved int32 = 64 bytes
    assert ctypes.sizeof(native.TbOptions) == 64
    # tb_plan_stats: 5 double, int64, 5 int32, 7 reserved = 96 bytes
    assert ctypes.sizeof(native.TbPlanStats) == 96
