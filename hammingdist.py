"""The reference's import name: ``import hammingdist`` gives this project's
GB300 implementation with the reference's Python API (ssciwr/hammingdist
1.4.0, python/hammingdist.cc:28-133: from_fasta, from_fasta_large,
from_fasta_to_lower_triangular, fasta_reference_distances,
fasta_sequence_indices, from_stringlist, from_csv, from_lower_triangular[_large],
distance, cuda_gpu_available, DataSet, DataSetLarge), so code written for the
reference runs unchanged. Every name is the one exported by hammingdist_gb300;
the distances are computed by its CUDA kernels, with no CPU path.
"""
from hammingdist_gb300 import (  # noqa: F401
    DataSet,
    DataSetLarge,
    cuda_gpu_available,
    distance,
    fasta_reference_distances,
    fasta_sequence_indices,
    from_csv,
    from_fasta,
    from_fasta_large,
    from_fasta_to_lower_triangular,
    from_lower_triangular,
    from_lower_triangular_large,
    from_stringlist,
)
# additions of this implementation (no reference counterpart)
from hammingdist_gb300 import (  # noqa: F401
    autotune,
    from_fasta_batch,
    from_fasta_device,
    load_tuning,
)
