"""The ctypes mirror of every C-ABI struct against the header itself: a C program compiled from
include/breseq_gb300.h prints each struct's size and each field's offset, which must equal the
ctypes layout (a mismatch would corrupt every call that passes the struct)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from breseq_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = {
    "Reference": "bsq_reference", "ReadSoA": "bsq_read_soa", "EcParams": "bsq_ec_params", "EcResult": "bsq_ec_result",
    "ImParams": "bsq_im_params", "RaRecord": "bsq_ra_record", "McRecord": "bsq_mc_record", "UnRecord": "bsq_un_record",
    "PositionArrays": "bsq_position_arrays", "RaSettings": "bsq_ra_settings", "RaCall": "bsq_ra_call",
    "CoverageFit": "bsq_coverage_fit", "ScParams": "bsq_sc_params", "ScSummary": "bsq_sc_summary",
    "ScPosition": "bsq_sc_position", "BamGroups": "bsq_bam_groups", "ReadArrays": "bsq_read_arrays",
    "CovColumns": "bsq_cov_columns", "Tuning": "bsq_tuning", "PairParams": "bsq_pair_params",
    "PdRegion": "bsq_pd_region", "PdSummary": "bsq_pd_summary", "PairRegion": "bsq_pair_region", "RaRaw": "bsq_ra_raw",
    "Job": "bsq_job", "JobInfo": "bsq_job_info", "ServerStats": "bsq_server_stats",
}


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "include/breseq_gb300.h"', "int main(void) {"]
    expect = []
    for py, cname in PAIRS.items():
        cls = getattr(abi, py)
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append((f"sizeof {cname}", C.sizeof(cls)))
        for name, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {name}));')
            expect.append((f"{cname}.{name}", getattr(cls, name).offset))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-I", ROOT, str(src), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    assert len(got) == len(expect)
    bad = [(k, v, g) for (k, v), g in zip(expect, got) if v != g]
    assert not bad, bad
