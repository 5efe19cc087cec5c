"""GB300-native IronClust clustering hot path: drift-constrained kNN, rho and
delta, behind a C ABI (libircgb300.so, include/ircgb300.h) that replaces the
reference's CUDA kernels argument for argument.

Modules:
  _lib      loads libircgb300.so and declares every C entry (ctypes)
  build     in-tree nvcc build of the library (sm_103a)
  irc       the MATLAB wrappers of the reference restated over the C ABI:
            drop-in kernels (search_min_drift, cuda_knn_index, ...), fused
            per-site plans (site_knn, site_delta, knn_rho_delta_site), the
            clustering that follows (sort_rho, assign_cluster_knn) and the
            on-device drift linkage (calc_drift)
  drift     chunk limits, linkage encoding and plan building (host logic of
            plan_sort_page_ / search_knn_drift_)
  batch     all sites of a probe as one plan over one feature matrix
  autotune  timed choice of the tensor-core work layout, cached per shape
  stream    a long recording paged from pinned FP16 host memory through a
            device ring of drift-chunk blocks
  files     the reference's on-disk formats (_fet_, _knn_, sort.irc)
  shard     site-to-rank assignment for one process per GPU
  synth     seeded synthetic sites and probes of the benchmark shapes
"""
