"""GB300-native INSCY subspace clustering (drop-in for the GPU run of mrjakobdk/GPU_INSCY)."""
from .inscy import GPU, GPU5, GPU_batch, clean_up, count_number_of_clusters, normalize, run_stats  # noqa: F401

__all__ = ["GPU", "GPU5", "GPU_batch", "normalize", "clean_up", "count_number_of_clusters", "run_stats"]
