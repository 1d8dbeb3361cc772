"""Test oracle for the separation likelihood (test infrastructure only; never
imported by the product library)."""
