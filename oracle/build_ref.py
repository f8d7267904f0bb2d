"""Recipe: compile TQP-Inmem's operator path into oracle/_ref/ (git-ignored build output).

    python oracle/build_ref.py [SOURCE_TREE]

SOURCE_TREE defaults to $TQP_REFERENCE, else /root/reference (where the TQP-Inmem tree is mounted
in the build container).  Nothing is copied: the modules are compiled into one bundle of code
objects (oracle/reference.py says which modules and how).  __graft_entry__.build() runs this when the
source tree is present; elsewhere (a GPU machine) the prebuilt oracle/_ref/ is used as it is.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

DEFAULT_SOURCE = "/root/reference"


def main(argv=None) -> Path | None:
    argv = sys.argv[1:] if argv is None else argv
    src = Path(argv[0] if argv else os.environ.get("TQP_REFERENCE", DEFAULT_SOURCE))
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    from oracle import reference
    if not (src / "operators" / "aggregate.py").exists():
        return reference.build(None)          # keep a previous build, if any
    return reference.build(src)


if __name__ == "__main__":
    print(main())
