"""Full-tensor potential solvers of ffthompy.tensorsLowRank (the low-rank
tensor formats themselves need ttpy and are not part of this package)."""
