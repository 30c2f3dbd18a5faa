"""The C-ABI library builds, loads and exports every entry point that
include/faco_gb300.h declares; host-only entry points work without a GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from gplsaco_gb300 import build, _lib
    build.build()
    return _lib.load()


def declared_functions():
    text = (ROOT / "include" / "faco_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(faco_\w+)\s*\(", text, re.M)))


def test_header_declarations_are_exported(lib):
    names = declared_functions()
    assert "faco_evaluate" in names and "faco_register_problem" in names
    for name in names:
        assert hasattr(lib, name), name
    from gplsaco_gb300 import _lib
    assert set(_lib.EXPORTED) == set(names)


def test_default_settings_match_reference_defaults(lib):
    from gplsaco_gb300 import _lib
    s = _lib.Settings()
    lib.faco_default_settings(C.byref(s))
    # cpp/include/gp_faco/fixed_faco_gpu.hpp:10-21
    assert (s.ants, s.primary_width, s.backup_width, s.ls_width) == (0, 16, 64, 20)
    assert (s.beta, s.retention, s.p_best, s.epoch_source_probability) == (1.0, 0.5, 0.1, 0.01)
    assert (s.ls_evaluation_limit, s.initial_ls_evaluation_limit) == (100000, 100000)


def _prog(**kw):
    p = dict(ir_version=1, numeric_spec_id=1, feature_spec_id=1, opcode=[0], operand=[4], constant_bits=[])
    p.update(kw)
    return p


@pytest.mark.parametrize("bad", [
    {"ir_version": 4},
    {"ir_version": True},
    {"opcode": [False]},
    {"operand": [4.0]},
    {"opcode": [0] + [7] * 6, "operand": [0] * 7},
    {"opcode": [0], "operand": [12]},
    {"opcode": [1], "operand": [0], "constant_bits": [0x7FC00000]},
    {"opcode": [0, 0, 3], "operand": [0, 1, 1]},
    {"opcode": [0, 0, 9], "operand": [0, 1, 0]},          # extended opcode under the reference grammar
])
def test_program_validation_rejects(lib, bad):
    # tests/python/test_native_scoring.py:57-68
    from gplsaco_gb300 import program_to_c
    with pytest.raises(ValueError):
        program_to_c(_prog(**bad))


def test_program_validation_accepts_and_matches_oracle(lib, oracle):
    from gplsaco_gb300 import _lib, program_to_c
    from tests import _programs
    rng = np.random.default_rng(1)
    for extended in (False, True):
        for _ in range(200):
            prog = _programs.random_program(rng, extended=extended)
            p = program_to_c(prog)
            assert lib.faco_validate_program(C.byref(p)) == _lib.FACO_OK
            assert oracle.lib().orc_validate_program(C.byref(oracle.program_struct(prog))) == 0


def test_settings_and_api_validation_without_gpu(lib):
    from gplsaco_gb300 import FixedFacoSettings
    with pytest.raises(ValueError):
        FixedFacoSettings(ants=True).to_c()
    with pytest.raises(ValueError):
        FixedFacoSettings(beta=float("nan")).to_c()
    assert FixedFacoSettings().to_c().ls_width == 20


def test_faco_ants_rule():
    from gplsaco_gb300 import faco_ants
    # python/gp_faco/worker.py:30-34
    assert [faco_ants(n) for n in (3, 256, 257, 1000, 1024, 1025, 10000)] == [64, 64, 128, 128, 128, 192, 448]
