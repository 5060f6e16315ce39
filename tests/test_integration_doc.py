"""INTEGRATION.md stays in step with the C header: the entry points and
constants its code blocks use are the ones include/kadath_gb300.h declares,
and its kd_newton_opts initializer names the struct's fields in their
order (a positional C initializer silently misassigns otherwise)."""
import re
from pathlib import Path

from test_abi_symbols import HEADER, declared_functions

DOC = Path(__file__).resolve().parent.parent / "INTEGRATION.md"


def code_blocks():
    text = DOC.read_text()
    return re.findall(r"```[a-z+]*\n(.*?)```", text, flags=re.S)


def test_documented_entry_points_and_constants_exist():
    header = HEADER.read_text()
    declared = set(declared_functions())
    defined = set(re.findall(r"#define\s+(KD_[A-Z0-9_]+)", header))
    used_f, used_c = set(), set()
    for block in code_blocks():
        used_f |= set(re.findall(r"\b(kd_[a-z0-9_]+)\s*\(", block))
        used_c |= set(re.findall(r"\b(KD_[A-Z0-9_]+)\b", block))
    assert used_f, "no entry point found in the code blocks"
    assert not sorted(used_f - declared), sorted(used_f - declared)
    assert not sorted(used_c - defined), sorted(used_c - defined)


def _struct_fields(name):
    header = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", header, flags=re.S).group(1)
    return re.findall(r"\b([a-z_][a-z0-9_]*)\s*;", body)


def test_newton_opts_initializer_follows_the_struct():
    fields = _struct_fields("kd_newton_opts")
    found = 0
    for block in code_blocks():
        m = re.search(r"kd_newton_opts\s+\w+\s*=\s*\{(.*?)\};", block, flags=re.S)
        if not m:
            continue
        found += 1
        named = re.findall(r"/\*\s*([a-z_][a-z0-9_]*)\s*\*/", m.group(1))
        assert named, "the initializer names no field"
        assert named == fields[:len(named)], (named, fields)
    assert found >= 1
