"""GB300-native engine for the RaySpace3D query path (point-in-mesh parity, filter-refine,
edge-ray overlap, containment fallback, pair dedup, grid selectivity estimator)."""
