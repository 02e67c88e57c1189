"""Where the reference checkout lies (test infrastructure).

One setting for every recipe that reads the reference's own sources or
example files: the environment variable PHYLOMMAND_REF, the root of a
phylommand checkout (holding src/ and example_files/).  Unset, it defaults to
the checkout this project was built against.  Where the directory does not
exist (e.g. on a GPU host), the recipes that need it skip themselves.
"""
from __future__ import annotations

import os

REF_ROOT = os.environ.get("PHYLOMMAND_REF", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")
REF_EXAMPLES = os.path.join(REF_ROOT, "example_files")


def have_sources() -> bool:
    return os.path.isdir(REF_SRC)


def have_examples() -> bool:
    return os.path.isdir(REF_EXAMPLES)
