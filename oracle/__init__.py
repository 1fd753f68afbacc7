"""Test oracle of the SW2D explicit step (test infrastructure, not product code)."""
