"""The per-entry-point kernel benchmark (lakcluster_c_gb300.kernel_bench)
names every entry point it times in its docstring, with the reference file
each replaces, and its command line accepts exactly those names."""
import pytest

from lakcluster_c_gb300 import kernel_bench as kb


def test_every_bench_is_documented():
    doc = kb.__doc__
    for name in kb.BENCHES:
        line = next(l for l in doc.splitlines() if l.strip().startswith(name + " ") or l.strip().startswith(name))
        assert "dir_c/" in line, name


def test_cli_rejects_unknown_names(monkeypatch):
    monkeypatch.setattr("sys.argv", ["kernel_bench", "--only", "no_such_kernel"])
    with pytest.raises(SystemExit):
        kb.main()
