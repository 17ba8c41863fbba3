"""Write tests/golden/reference_kats.json (and copy the reference's HDF5 test file).

The reference (ITensors.jl / NDTensors.jl, Julia) cannot run here (there is no
Julia toolchain), and its test suite stores no numeric golden vectors for the
contraction path.  Its known-answer tests are literals inside the Julia test
files; this script records those literals, each with the file:line it comes
from, so the oracle can be pinned against them.  Only the reference's stated
expectations are recorded here (no value computed by this project).

Run:  python tests/golden/make_golden.py
"""
import json
from pathlib import Path

KATS = {
    "truncate": [
        {"src": "test/base/test_decomp.jl:96-99", "P": [0.1, 0.01, 1.0e-13],
         "kwargs": {"use_absolute_cutoff": True, "cutoff": 1.0e-5},
         "truncerr": 1.0e-13, "docut": (0.01 + 1.0e-13) / 2, "len": 2},
        {"src": "test/base/test_decomp.jl:103-105", "P": [-0.12, -0.1], "kwargs": {},
         "truncerr": 0.0, "docut": 0.0, "len": 2},
        {"src": "test/base/test_decomp.jl:107-110", "P": [-0.1, -0.01, -1.0e-13],
         "kwargs": {"use_absolute_cutoff": True, "cutoff": 1.0e-5},
         "truncerr": 1.0e-13, "docut": (0.01 + 1.0e-13) / 2, "len": 2},
    ],
    "blocksparse_structure": {
        "src": "NDTensors/test/test_blocksparse.jl:27-39",
        "inds": [[2, 3], [4, 5]], "blocks": [[1, 2], [2, 1]],
        "blockdims": {"1,2": [2, 5], "2,1": [3, 4]}, "nnz": 22, "nnzblocks": 2,
    },
    "blocksparse_permutedims": {
        "src": "NDTensors/test/test_blocksparse.jl:101-110",
        "inds": [[2, 3], [4, 5]], "blocks": [[1, 2], [2, 1]], "perm": [2, 1],
        "blockdims_after": {"1,2": [4, 3], "2,1": [5, 2]}, "nnz": 22,
    },
    "insert_blocks_nnz": {
        "src": "NDTensors/test/test_blocksparse.jl:222-274",
        "inds": [[2, 3], [4, 5]], "insert_order": [[1, 1], [2, 2], [1, 2], [2, 1]],
        "nnz_sequence": [8, 23, 33, 45],
    },
    "qn_contraction": {
        "src": "test/base/test_qnitensor.jl:564-583",
        "i": [[0, 1], [1, 2]], "j": [[0, 3], [1, 4]],
        "A": {"inds": ["i", "dag(j)"], "flux": 0, "nnzblocks": 2},
        "B": {"inds": ["j", "dag(i)'"], "flux": 1, "nnzblocks": 1},
        "C": {"nnzblocks": 1, "flux": 1},
    },
    "flux_docstring": {
        "src": "src/indexset.jl:866-873",
        "i": [[0, 2], [1, 2]], "inds": ["i", "dag(i')"],
        "flux": {"1,1": 0, "2,1": 1, "1,2": -1, "2,2": 0},
    },
    "multithreading_doc": {
        "src": "docs/src/Multithreading.md:105-108 (A' * B, order 4, each index [QN(0)=>20, QN(1)=>20])",
        "d": 20, "pairs": 10, "flops": 2 * 10 * 20 ** 6,
    },
    "threaded_no_blocks": {
        "src": "test/threading/test_threading.jl:60-78",
        "i": [[0, 1], [1, 1]], "A_block": [1, 1], "B_block": [2, 2],
        "nnzblocks": 0, "nnz": 0,
    },
    "threaded_contraction": {
        "src": "test/threading/test_threading.jl:30-41",
        "i": [[0, 500], [1, 500]], "R_equals_threaded": True,
    },
    "svd_min_blockdim": {
        "src": "test/base/test_decomp.jl:469-491",
        "i": [[4, 1], [2, 4], [0, 6], [-2, 4], [-4, 1]], "cutoff": 1.0e-1, "min_blockdim": 2,
    },
    "nan_overwrite": {
        "src": "NDTensors/test/test_dense.jl:237-259",
        "R_dims": [2, 2, 1], "T1_dims": [2, 2, 1], "T2_dims": [1, 1],
        "labels_noperm": {"R": [1, 2, 3], "T1": [1, 2, -1], "T2": [-1, 1]},
        "labels_perm": {"R": [2, 1, 3], "T1": [1, 2, -1], "T2": [-1, 1]},
    },
}

# HDF5 file written by the reference through libhdf5 (an ITensor with Dense{Float64}
# storage), the fixture of its test/base/test_readwrite.jl:182-190; it pins the HDF5
# reader of the package's BlockSparse storage I/O.
HDF5_FIXTURE = ("test/base/utils/testfilev0.1.41.h5", "itensor_v0.1.41_dense.h5")

if __name__ == "__main__":
    out = Path(__file__).with_name("reference_kats.json")
    out.write_text(json.dumps(KATS, indent=1) + "\n")
    print(out)
    import shutil
    src = Path("/root/reference") / HDF5_FIXTURE[0]
    if src.exists():
        dst = Path(__file__).with_name(HDF5_FIXTURE[1])
        shutil.copyfile(src, dst)
        print(dst)
