"""Where the reference checkout lies, for the tests and scripts that read its
sources: $NWG_REFERENCE when set, else a directory named `reference` beside
this repository.  Tests that need it skip when neither exists (the reference
never travels with the repository)."""
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("NWG_REFERENCE") or os.path.normpath(os.path.join(ROOT, os.pardir, "reference"))


def present(name: str = "SpeciesBlock.cpp") -> bool:
    return os.path.isfile(os.path.join(REF, name))
