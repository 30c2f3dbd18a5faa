"""Random GP programs for the tests (the generator lives in the package)."""
from gplsaco_gb300.programs import EXTENDED_OPS, REFERENCE_OPS, random_program  # noqa: F401
