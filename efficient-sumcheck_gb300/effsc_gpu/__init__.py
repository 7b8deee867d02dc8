"""effsc_gpu -- GB300 sumcheck prover behind the effsc crate's API.

The compute path is the CUDA library ``_build/libeffsc_gpu.so`` (sm_103a);
this package is its ctypes front end.  See include/effsc_gpu.h for the C ABI.
"""
from ._lib import EffscError, ReferencePanic, LIB_PATH, load  # noqa: F401
from .api import (  # noqa: F401
    CANONICAL, COEF, EQF, FP, FP3, GKR, IP, LSB, ML, MONTGOMERY, MSB, T_KECCAK, T_TEST,
    Batch, CoefficientProver, CoefficientSumcheck, Evaluator, coefficient_sumcheck, pw_even, pw_odd, tw_even,
    tw_odd, GkrProver, CoefficientProverLSB, Context, EqFactoredProver, InnerProductProver,
    InnerProductProverLSB, MultilinearProver, MultilinearProverLSB, ProductSumcheck, Server, Sumcheck,
    SumcheckProof, Transcript, build_eq_table, compute_sumcheck_polynomial, fold,
    fused_fold_and_compute_polynomial, gen_uniform, inner_product_sumcheck,
    inner_product_sumcheck_partial, launch_count, launch_count_reset, multilinear_sumcheck,
    multilinear_sumcheck_partial, noop_hook, sumcheck, sumcheck_verify, sumcheck_verify_batch, table_seed,
    protogalaxy_fold, protogalaxy_fold_raw,
    FileStream, MemoryStream, multivariate_claim, multivariate_product_claim, reorder_vec_msb,
)
