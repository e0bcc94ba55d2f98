"""CPU oracle for the M-plicits nested sine-MLP hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, on the CPU, the reference
algorithm the GPU library accelerates, so that the GPU results can be
checked.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
CPU-baseline leg, its reference arm and its error statement) may import it,
and only as the checker: the product path in ``mplicits_gb300`` never calls
into it and has no CPU fallback.

Modules
-------
siren     numpy FP32/FP64 evaluator of ``i3d.model.SIREN`` and the grid of
          ``i3d.meshing.gen_mc_coordinate_grid`` (division quirk included),
          the band-culled loop of ``i3d.meshing.create_mesh_multistage`` and
          ``reconstruct.adaptive_deltas``.
mc        ctypes wrapper of ``mc.c``: marching cubes with the derived case
          table and a canonical vertex/face order (the reference uses
          scikit-image, which is absent here: parity to scikit-image itself is
          unpinned; the GPU kernel is pinned to this restatement).
fp64      torch FP64 evaluator used only to state the SDF error of results.
deltas    ctypes wrapper of ``deltas.c``: calc_deltas
          (experiment_scripts/utils.py:46-89) over an exact float32
          nearest-triangle distance, brute force or on a uniform grid (open3d,
          whose scene the reference queries, is absent: parity to its rounding
          is unpinned; the loop is pinned to the reference's own code).

Pinning: ``tests/golden`` holds vectors generated by importing the reference
``i3d`` package (``tests/golden/make_golden.py``); ``tests/test_oracle.py``
checks this oracle against them.
"""
