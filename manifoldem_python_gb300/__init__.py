"""GB300-native (sm_103a) per-projection-direction CTF-distance stage of ManifoldEM.

Drop-in modules: ``getDistanceCTF_local_Conj9combinedS2`` (per-PD ``op``), ``GetDistancesS2``
(driver), ``p``, ``myio``, ``set_params``.  Batched API: ``pipeline.DistanceStage``.
The compute path is the CUDA library built from ``csrc/`` (``_lib.build()``).
"""
__version__ = '0.1.0'
