"""Command line interface: flags and errors (CPU), and the reference's own
output format on the golden 1AMY / 1.3.3 case (GPU)."""

import io
import shutil

import pytest

from helpers import parse_block


def test_parser_flags():
    from pyjess_gb300.cli import argument_parser, ignore_chain_mode

    p = argument_parser()
    a = p.parse_args(["-T", "t", "-Q", "q", "-R", "2", "-D", "3", "-M", "4"])
    assert (a.rmsd, a.distance_cutoff, a.maximum_distance) == (2.0, 3.0, 4.0)
    assert a.transform and a.reorder and not a.best_match and a.max_candidates is None
    assert ignore_chain_mode(a) is None
    a = p.parse_args(["-T", "t", "-Q", "q", "-R", "2", "-D", "3", "-M", "4", "-n", "--no-reorder", "-b",
                      "-c", "7", "--ignore-res-chain"])
    assert not a.transform and not a.reorder and a.best_match and a.max_candidates == 7
    assert ignore_chain_mode(a) == "residues"
    a = p.parse_args(["-T", "t", "-Q", "q", "-R", "2", "-D", "3", "-M", "4", "-i", "--ignore-res-chain"])
    assert ignore_chain_mode(a) == "atoms"
    with pytest.raises(SystemExit):
        p.parse_args(["-T", "t"])


def test_version(capsys):
    from pyjess_gb300 import __version__
    from pyjess_gb300.cli import main

    with pytest.raises(SystemExit):
        main(["-V"])
    assert __version__ in capsys.readouterr().out


def test_missing_template_list_is_an_error(tmp_path):
    from pyjess_gb300.cli import main

    out, err = io.StringIO(), io.StringIO()
    rc = main(["-T", str(tmp_path / "none.list"), "-Q", str(tmp_path / "q.list"), "-R", "2", "-D", "2", "-M", "2"],
              stdout=out, stderr=err)
    assert rc != 0 and err.getvalue().startswith("Error: ") and out.getvalue() == ""


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 4])
def test_cli_golden_1amy(tmp_path, monkeypatch, golden, golden_blocks, batch):
    """Jess's own output for 1AMY against template 1.3.3 (named template.pdb
    there): same hits in the same order, same fields within the file's
    precision, through the batched CLI (the molecule listed three times)."""
    from pyjess_gb300.cli import main

    shutil.copy(golden / "1.3.3.tpl", tmp_path / "template.pdb")
    (tmp_path / "templates.list").write_text("template.pdb\n")
    (tmp_path / "queries.list").write_text(f"{golden / '1AMY.pdb'}\n" * 3)
    monkeypatch.chdir(tmp_path)
    out, err = io.StringIO(), io.StringIO()
    rc = main(["-T", "templates.list", "-Q", "queries.list", "-R", "2", "-D", "4", "-M", "4", "--no-reorder",
               "--batch", str(batch)], stdout=out, stderr=err)
    assert rc == 0, err.getvalue()
    blocks = [b for b in out.getvalue().split("REMARK") if b.strip()]
    assert len(blocks) == 3 * len(golden_blocks) == 3 * 156
    for got, want in zip(blocks, golden_blocks * 3):
        gid, grmsd, gdet, gloge, glines = parse_block(got)
        wid, wrmsd, wdet, wloge, wlines = parse_block(want)
        assert gid == wid == "1AMY"
        assert got.strip().splitlines()[0].split()[2] == "template.pdb"
        assert grmsd == pytest.approx(wrmsd, abs=1e-3)
        assert gdet == pytest.approx(wdet, abs=0.05)
        assert gloge == pytest.approx(wloge, abs=0.011)
        assert len(glines) == len(wlines)
        for gl, wl in zip(glines, wlines):
            assert gl[:30] == wl[:30]
            for c0, c1 in ((30, 38), (38, 46), (46, 54)):
                assert float(gl[c0:c1]) == pytest.approx(float(wl[c0:c1]), abs=1.5e-3)


@pytest.mark.parametrize("codec", ["gzip", "bz2", "lzma", None])
def test_zopen_decompresses_by_magic(tmp_path, codec):
    import importlib

    from pyjess_gb300.cli import zopen

    text = "template.pdb\nother.pdb\n"
    path = tmp_path / "list.txt"
    if codec is None:
        path.write_text(text)
    else:
        with importlib.import_module(codec).open(path, "wt") as f:
            f.write(text)
    with zopen(path) as f:
        assert f.read() == text
