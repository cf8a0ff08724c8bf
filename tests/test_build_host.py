"""The in-tree build's staleness rules (graspan-g_gb300/build.py), with the compilers
replaced by a recorder that touches the outputs: a second build with the same flags
compiles nothing, and a build with other NVCC overrides (GRG_NVCC_DEFS, e.g. a tuning
A/B) recompiles every CUDA source. No GPU or compiler runs."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load_build(monkeypatch, out, defs):
    monkeypatch.setenv("GRG_BUILD_DIR", str(out))
    monkeypatch.setenv("GRG_NVCC_DEFS", defs)
    spec = importlib.util.spec_from_file_location("grg_build_under_test",
                                                  os.path.join(ROOT, "graspan-g_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    ran = []

    def fake_run(cmd):
        ran.append(cmd)
        out_path = cmd[cmd.index("-o") + 1]
        with open(out_path, "w") as f:
            f.write("x")
        return ""

    monkeypatch.setattr(mod, "_run", fake_run)
    monkeypatch.setattr(mod, "_nvcc", lambda: "nvcc")
    return mod, ran


def _compiled(ran):
    return sorted(os.path.basename(c[c.index("-c") + 1]) for c in ran if "-c" in c)


def test_rebuild_only_when_sources_or_overrides_change(tmp_path, monkeypatch):
    out = tmp_path / "build"
    mod, ran = _load_build(monkeypatch, out, "")
    mod.build()
    first = _compiled(ran)
    assert "grg_engine.cu" in first and "grg_format.cu" in first
    mod, ran = _load_build(monkeypatch, out, "")
    mod.build()
    assert _compiled(ran) == []                       # nothing changed: nothing compiled
    mod, ran = _load_build(monkeypatch, out, "-DGRG_WIN2=16 -DGRG_WIN2_LO=8")
    mod.build()
    assert set(_compiled(ran)) >= {"grg_engine.cu", "grg_format.cu"}    # new overrides: recompiled
    assert any("-DGRG_WIN2=16" in c for c in ran)
    mod, ran = _load_build(monkeypatch, out, "-DGRG_WIN2=16 -DGRG_WIN2_LO=8")
    mod.build()
    assert _compiled(ran) == []
