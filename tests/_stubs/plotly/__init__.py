"""Minimal stand-in so the reference package imports without plotly (tests only)."""
