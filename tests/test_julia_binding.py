"""Static checks of the Julia binding flowvpm.jl_gb300/julia/UJ_gb300.jl (CPU).

No Julia toolchain exists here, so the file cannot run; these checks keep it
consistent with the C ABI and with the Python mirror that the GPU tests run:

* every `ccall((:vpm_..., libvpm), ...)` names a function declared in
  include/vpm_gb300.h and passes as many arguments as its prototype has;
* the drop-in hook `_uj` takes the keywords of UJ_direct
  (src/FLOWVPM_UJ.jl:21-25) -- rbf, sfs, reset, reset_sfs -- with the same
  defaults as vpm_gb300.uj.UJ_gb300, and accepts rbf=true (ignored, as
  UJ_direct does);
* the ChainRulesCore rules are in the file (not only in documentation): one for
  the UJ core over vpm_uj_adjoint_dev and one for the Estr core over
  vpm_estr_adjoint_dev.
"""
import inspect
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "flowvpm.jl_gb300", "julia", "UJ_gb300.jl")
HDR = os.path.join(ROOT, "include", "vpm_gb300.h")


def _split_top(s):
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _matching(s, i):
    """Index of the bracket closing the one at s[i]."""
    depth = 0
    for j in range(i, len(s)):
        if s[j] in "({[":
            depth += 1
        elif s[j] in ")}]":
            depth -= 1
            if depth == 0:
                return j
    raise ValueError("unbalanced")


def _prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(?:int|int64_t|const char\s*\*)\s+(vpm_\w+)\s*\(", src):
        j = _matching(src, m.end() - 1)
        args = src[m.end():j].strip()
        protos[m.group(1)] = 0 if args in ("", "void") else len(_split_top(args))
    return protos


def _ccalls():
    src = open(JL).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(\w+), libvpm\),\s*\w+,\s*", src):
        i = m.end()
        assert src[i] == "(", m.group(1)
        j = _matching(src, i)
        types = _split_top(src[i + 1:j])
        k = src.index(",", j) + 1
        end = _matching(src, m.start() + len("ccall"))
        args = _split_top(src[k:end])
        calls.append((m.group(1), types, args))
    return calls


def test_every_ccall_matches_a_header_prototype():
    protos = _prototypes()
    calls = _ccalls()
    assert len(calls) >= 10
    for name, types, args in calls:
        assert name in protos, name
        assert len(types) == protos[name], (name, len(types), protos[name])
        assert len(args) == len(types), (name, len(args), len(types))


def test_drop_in_keywords_match_the_python_mirror():
    import vpm_gb300.uj as uj
    src = open(JL).read()
    m = re.search(r"function _uj\(pfield, precision::Cint;(.*?)\)\n", src, flags=re.S)
    jl = dict(re.findall(r"(\w+)::Bool=(\w+)", m.group(1)))
    py = {k: str(v.default).lower() for k, v in inspect.signature(uj.UJ_gb300).parameters.items()
          if k in ("rbf", "sfs", "reset", "reset_sfs")}
    assert jl == py
    assert "rbf && error" not in src        # rbf=true is accepted, as UJ_direct accepts it


def test_rrules_are_in_the_binding():
    src = open(JL).read()
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(uj_gb300_core\)", src)
    assert re.search(r"function ChainRulesCore\.rrule\(::typeof\(estr_gb300_core\)", src)
    names = {c[0] for c in _ccalls()}
    assert {"vpm_uj_adjoint_dev", "vpm_estr_adjoint_dev", "vpm_uj_dev", "vpm_estr_dev", "vpm_uj"} <= names
