"""Where the reference tree (opensbli, read-only) is found by the oracle's generation recipes.

Test infrastructure.  The location comes from the OPENSBLI_REFERENCE environment variable; without
it, a directory named `reference` beside the repository's root directory is used.
"""
import os

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def default_ref():
    return os.environ.get("OPENSBLI_REFERENCE") or os.path.normpath(os.path.join(REPO, "..", "reference"))
