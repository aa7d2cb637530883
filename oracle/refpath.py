"""Test infrastructure: where the reference tree lies, for the checker's
recipes that read it (the golden-fixture scripts and the tests that compare
with the reference compiled from source).  Override with BD_REFERENCE_ROOT;
the GPU host has no reference tree, and nothing that runs there reads it."""
import os

REF_ROOT = os.environ.get("BD_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "BD_cuda")
REF_TESTDATA = os.path.join(REF_ROOT, "test_data")
