"""Copy the reference's own test fixtures into ``tests/golden/``.

The reference keeps its golden vectors as data files next to its unit tests
(``src/pyjess/tests/data`` of the PyJess source tree).  The GPU test machine
does not have the reference checkout, so the files the parity tests need are
committed here.  Run this script once with the path of a PyJess checkout::

    python tests/golden/make_fixtures.py <pyjess-source-tree>

Files copied (all used by the parity tests):

- ``1AMY.pdb``        barley alpha-amylase, 3,339 atoms (ATOM + HETATM)
- ``1.3.3.tpl``       9-atom M-CSA template (modes 1 and 3)
- ``4.1.2.tpl``       9-atom M-CSA template (modes 0, 1 and 3)
- ``1sur.qry``        12-atom two-chain template (dimension test)
- ``5ayx.EF.pdb``     two-chain fragment for the ``ignore_chain`` tests
- ``1AMY+1.3.3.txt``  Jess's own output, 156 hits in scanner order
- ``1AMY.cif``        the same structure in mmCIF (the mmCIF reader's tests)
"""

import argparse
import pathlib
import shutil

DATA = pathlib.Path("src/pyjess/tests/data")
FILES = ["1AMY.pdb", "1.3.3.tpl", "4.1.2.tpl", "1sur.qry", "5ayx.EF.pdb", "1AMY+1.3.3.txt", "1AMY.cif"]


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("source", type=pathlib.Path, help="root of a PyJess source tree")
    args = ap.parse_args()
    here = pathlib.Path(__file__).parent
    for name in FILES:
        shutil.copyfile(args.source / DATA / name, here / name)
        print("copied", name)


if __name__ == "__main__":
    main()
