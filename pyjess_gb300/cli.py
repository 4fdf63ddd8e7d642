"""Command line interface with the flags and output of PyJess's ``pyjess``
(``src/pyjess/cli.py:84-283``).

Templates and queries come from list files (one path per line, as in the
reference), hits are written to stdout as PDB blocks (`Hit.dump`, one blank
line after each), in query order and, per query, in the order ``query()``
yields them.  The difference is in how the search runs: query molecules are
parsed by a pool of host threads (``--jobs``; the reference accepts the flag
but searches one molecule at a time) and searched ``--batch`` molecules at a
time in one batched device query (`Jess.query_many`), instead of one
`Jess.query` per molecule.
"""

from __future__ import annotations

import argparse
import concurrent.futures
import contextlib
import io
import os
import sys
import typing
import warnings
from pathlib import Path

from . import __version__
from ._jess import Jess, Molecule, Template

_BZ2_MAGIC = b"BZh"
_GZIP_MAGIC = b"\x1f\x8b"
_XZ_MAGIC = b"\xfd7zXZ"


@contextlib.contextmanager
def zopen(path, mode="r", encoding=None, errors=None, newline=None) -> typing.Iterator[typing.IO]:
    """Open a file, decompressing gzip, bzip2 or xz by its magic bytes
    (``src/pyjess/cli.py:52-81``; lz4 and zstd need modules that are not
    installed here and are reported as errors)."""
    with contextlib.ExitStack() as ctx:
        file = ctx.enter_context(open(path, "rb"))
        peek = file.peek()
        if peek.startswith(_GZIP_MAGIC):
            import gzip
            file = ctx.enter_context(gzip.open(file, mode="rb"))
        elif peek.startswith(_BZ2_MAGIC):
            import bz2
            file = ctx.enter_context(bz2.open(file, mode="rb"))
        elif peek.startswith(_XZ_MAGIC):
            import lzma
            file = ctx.enter_context(lzma.open(file, mode="rb"))
        elif peek.startswith(b"\x04\x22\x4d\x18"):
            raise RuntimeError("File compression is LZ4 but lz4 is not installed")
        elif peek.startswith(b"\x28\xb5\x2f\xfd"):
            raise RuntimeError("File compression is ZSTD but zstandard is not installed")
        if mode == "r":
            file = io.TextIOWrapper(file, encoding=encoding, errors=errors, newline=newline)
        yield file


def argument_parser(prog: str = "pyjess", version: str = __version__) -> argparse.ArgumentParser:
    parser = argparse.ArgumentParser(
        prog=prog,
        add_help=False,
        formatter_class=argparse.RawDescriptionHelpFormatter,
        description="PyJess on GB300 - 3D template matching against many structures at once.",
    )
    parser.add_argument("-h", "--help", action="help", help="Show this help message and exit.")
    parser.add_argument("-V", "--version", action="version", version=f"PyJess {version}",
                        help="Show the version number and exit.")
    parser.add_argument("-j", "--jobs", type=int, default=os.cpu_count() or 1,
                        help="The number of threads parsing query files.")
    parser.add_argument("--batch", type=int, default=256,
                        help="Query molecules searched together in one device query.")
    parser.add_argument("--precision", choices=("fp32", "fp64"), default="fp32",
                        help="Distance tests in FP32 with a guard band and FP64 recheck, or in FP64.")

    group = parser.add_argument_group("Mandatory Parameters")
    group.add_argument("-T", "--templates", type=Path, required=True, help="The path to the template list file.")
    group.add_argument("-Q", "--queries", type=Path, required=True, help="The path to the query list file.")
    group.add_argument("-R", "--rmsd", type=float, required=True, help="The RMSD threshold.")
    group.add_argument("-D", "--distance-cutoff", type=float, required=True, help="The distance-cutoff.")
    group.add_argument("-M", "--maximum-distance", type=float, required=True,
                       help="The maximum allowed template/query atom distance after adding the global distance "
                            "cutoff and the individual atom distance cutoff defined in the temperature field of "
                            "the ATOM record in the template file.")

    group = parser.add_argument_group("Flags")
    group.add_argument("-n", "--no-transform", action="store_false", dest="transform",
                       help="Do not transform coordinates of hit into the template coordinate frame")
    group.add_argument("-f", "--filenames", action="store_true", help="Show PDB filenames in progress on stderr")
    group.add_argument("-i", "--ignore-chain", action="store_true",
                       help="Include matches composed of residues belonging to multiple chains (if template is "
                            "single-chain) or matches with residues from a single chain (if template has "
                            "residues from multiple chains).")
    group.add_argument("--ignore-res-chain", action="store_true",
                       help="Include matches composed of residues belonging to multiple chains but still "
                            "enforce all atoms of a residue to be part of the same chain.")
    group.add_argument("-q", "--query-filename", action="store_true",
                       help="Write filename of query instead of PDB ID from HEADER")
    group.add_argument("-e", "--ignore-endmdl", action="store_true",
                       help="Parse atoms from all models separated by ENDMDL (use with care).")
    group.add_argument("-c", "--max-candidates", type=int, default=None,
                       help="Set a maximum number of candidates to return by template.")
    group.add_argument("--no-reorder", action="store_false", dest="reorder",
                       help="Disable template atom reordering in the matching process, so results come in the "
                            "same order as the original Jess.")
    group.add_argument("-b", "--best-match", action="store_true",
                       help="Return only the best match for each template/query pair.")
    return parser


def ignore_chain_mode(args) -> typing.Optional[str]:
    """The `ignore_chain` mode of the flags; ``-i`` wins over
    ``--ignore-res-chain``.  The reference passes ``"all"`` for ``-i``
    (``cli.py:248``), which its own `Query` rejects as invalid; the mode the
    flag describes is ``"atoms"``, used here."""
    return "atoms" if args.ignore_chain else "residues" if args.ignore_res_chain else None


def _load_query(filename: str, args) -> Molecule:
    id_ = filename if args.query_filename else None
    mol = Molecule.load(filename, id=id_, ignore_endmdl=args.ignore_endmdl)
    if mol.id is None:
        warnings.warn(f"No id in molecule {filename}. Using filename instead.")
        mol = Molecule(mol, id=filename, date=mol.date, name=mol.name)
    return mol


def main(argv: typing.Optional[typing.List[str]] = None, stdout: typing.TextIO = sys.stdout,
         stderr: typing.TextIO = sys.stderr) -> int:
    parser = argument_parser()
    args = parser.parse_args(argv)
    ignore_chain = ignore_chain_mode(args)
    if args.batch < 1:
        print("Error: --batch must be at least 1", file=stderr)
        return 1

    try:
        with args.templates.open() as f:
            templates = [Template.load(n, id=n) for n in map(str.strip, f)]
        jess = Jess(templates)
        with args.queries.open() as f:
            filenames = [line.strip() for line in f]
        jobs = max(1, args.jobs)
        with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as pool:
            for b0 in range(0, len(filenames), args.batch):
                names = filenames[b0:b0 + args.batch]
                molecules = list(pool.map(lambda n: _load_query(n, args), names))
                per = jess.query_many(molecules, args.rmsd, args.distance_cutoff, args.maximum_distance,
                                      max_candidates=args.max_candidates, ignore_chain=ignore_chain,
                                      reorder=args.reorder, best_match=args.best_match,
                                      precision=args.precision)
                for filename, hits in zip(names, per):
                    if args.filenames:
                        print(filename, file=stderr)
                    for hit in hits:
                        hit.dump(stdout, format="pdb", transform=args.transform)
                        stdout.write("\n")
    except Exception as err:
        print("Error: {}".format(err), file=stderr)
        return getattr(err, "errno", None) or 1
    return 0
