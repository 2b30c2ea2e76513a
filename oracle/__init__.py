"""CPU oracle of the meshlet raster pipeline (test infrastructure; see oracle.py)."""
