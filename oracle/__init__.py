"""Test infrastructure: CPU oracle (liboracle.so) and the reference driver (_ref/libbdref.so)."""
