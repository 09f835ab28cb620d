"""The C ABI library: it loads without a GPU and exports every entry point
include/ntp.h declares; the ctypes records match the header's sizes."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from neutrinotelescopes_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]


def header_functions() -> set[str]:
    text = (ROOT / "include" / "ntp.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(ntp_[a-z_0-9]+)\s*\(", text))


def test_header_matches_python_list():
    assert header_functions() == set(_abi.EXPORTED)


def test_library_exports_every_symbol():
    lib = _abi.load_library()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.ntp_abi_version() == _abi.NTP_ABI_VERSION


def test_nm_lists_symbols():
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(_abi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ntp_\w+)", out))
    assert header_functions() <= exported


def test_record_layouts():
    assert C.sizeof(_abi.NtpSource) == 64
    assert C.sizeof(_abi.NtpTarget) == 48
    assert _abi.HIT_DTYPE.itemsize == 64
    assert _abi.HIT_DTYPE.fields["module_id"][1] == 48
    assert _abi.HIT_DTYPE.fields["photon_index"][1] == 56
    assert _abi.NtpSource.photons.offset == 32
    assert _abi.NtpMediumDesc.hg_g.offset == 64
    # ntp_flow_config: 3 int32, 8 floats (t_min .. count_weight), then the u64 seed
    assert _abi.NtpFlowConfig.count_weight.offset == 40
    assert _abi.NtpFlowConfig.seed.offset == 48
    assert C.sizeof(_abi.NtpFlowConfig) == 64


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="missing"):
        _abi.load_library(tmp_path / "libntp.so")


def test_create_without_gpu_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = _abi.load_library()
    ctx = C.c_void_p()
    st = lib.ntp_create(0, C.byref(ctx))
    assert st != _abi.NTP_OK and not ctx.value
    assert lib.ntp_last_error(None)


# (C struct in include/ntp.h, ctypes mirror) pairs checked field by field
_RECORDS = [("ntp_source", "NtpSource"), ("ntp_target", "NtpTarget"), ("ntp_medium_desc", "NtpMediumDesc"),
            ("ntp_spectrum_desc", "NtpSpectrumDesc"), ("ntp_prop_opts", "NtpPropOpts"),
            ("ntp_run_stats", "NtpRunStats"), ("ntp_summary_spec", "NtpSummarySpec"),
            ("ntp_table_spec", "NtpTableSpec"), ("ntp_flow_config", "NtpFlowConfig"),
            ("ntp_server_config", "NtpServerConfig"), ("ntp_event_result", "NtpEventResult"),
            ("ntp_server_stats", "NtpServerStats")]


def test_ctypes_records_match_the_header(tmp_path):
    """Every ctypes record has the size and field offsets that a C compiler
    gives the header's struct (compiled with gcc here)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ntp.h"', "int main(void) {"]
    expect = {}
    for cname, pyname in _RECORDS:
        cls = getattr(_abi, pyname)
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        expect[f"{cname} size"] = C.sizeof(cls)
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
            expect[f"{cname} {fname}"] = getattr(cls, fname).offset
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        key, val = line.rsplit(" ", 1)
        got[key] = int(val)
    assert got == expect
