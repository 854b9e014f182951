"""Preconditioners for the CG(P=...) hook: the learned FSAI factor (learned_fsai)."""
