"""Constants of the dense hot path, one place.

Values that the reference fixes are mirrored from its ``src/mbem/defaults.py``
(line numbers in the comments) so that a result here is comparable with the
reference's at the same settings; GPU-only settings follow.
"""

# ---- solver (defaults.py:10-17) ----
SOLUTION_RTOL = 1e-6
GMRES_RTOL = 1e-8
GMRES_RESTART = 200
GMRES_MAXITER = 600
GMRES_STAGNATION_WINDOW = 100
GMRES_STAGNATION_FACTOR = 10.0
COND_WARN_THRESHOLD = 1e10            # defaults.py:118

# ---- eps (defaults.py:798-808) ----
EPS_OVER_H = 0.1
FAULT_EPS_OVER_H = 0.07
HALF_JUMP_MAX_EPS_OVER_H = 0.5

# ---- readout (defaults.py:846) ----
EIGEN_NEAR_RADIUS_EPS = 20.0
NEAR_BOUNDARY_H_RATIO = 0.5

# ---- volume sampler (defaults.py:833) ----
VOLUME_CHUNK = 50_000                 # the reference's chunk (host memory bound)
VOLUME_CHUNK_DEVICE = 1 << 18         # points a readout launch takes here (~100 MB of device state)

# ---- nodal kernels (defaults.py:916-932) ----
NODAL_D_STAR = 10.0
NODAL_FAR_GAUSS_N = 12
NODAL_FAR_GAUSS_N_DISTANT = 8
NODAL_D_STAR_DISTANT = 40.0
NODAL_SERIES_U_OVER_RHO = 2.0
NODAL_SERIES_TERMS = 32
NODAL_SMALL_U_OVER_RHO = 0.5
NODAL_MIN_HEIGHT_OVER_L = 1e-3

# ---- layout (defaults.py:957-981) ----
COLLOCATION_SHRINK_BY_ORDER = {0: 0.0, 1: 0.5, 2: 0.5}
COLLOCATION_FAULT_CLEARANCE_EPS = 1.0
FRAME_FLAT_TOL = 1e-12
MIN_TRIANGLE_HEIGHT_OVER_L = 1e-6
TRACTION_VALUE_NORMAL_TOL = 1e-12

# ---- block-Jacobi preconditioner (defaults.py:712) ----
PRECOND_BJ_CHUNK_DOF = 9000

# ---- dense LU (defaults.py:1243-1261) ----
LU_REFINE_TOL = 1.0e-10                # stop when what is left after a correction is this small
LU_REFINE_PASSES = 4                   # at most this many corrections
LU_REFINE_RATE = 1.0e-2                # corrections that contract worse than this: not single-precision material

# ---- GPU mixed-precision path ----
MIXED_BLOCK = 64                      # BF16 scale block (rows x columns)
MIXED_NEAR_RADIUS_FACTOR = 3.0        # near field: centroid distance < 3 max(eps, h)
MIXED_INNER_ITERATIONS = 40           # at most this many BF16 inner GMRES steps per outer step
MIXED_INNER_RTOL = 1e-5               # ... or until the inner residual estimate is this small

# ---- compressed pair operator (defaults.py:128-320 of the reference) ----
BLOCK_COMPRESSION_TOL = 1e-4           # relative Frobenius tolerance of an admissible block
CLUSTER_MIN_LEAF = 96                  # cluster-tree leaves hold at most this many elements
ADMISSIBILITY_ETA = 2.0                # admissible: min(diam_f, diam_s) < eta * dist(box_f, box_s)
ACA_MIN_BLOCK = 64                     # admissible blocks with a side below this are dense
MAX_ADMISSIBLE_BLOCK = 1024            # admissible blocks have at most this many elements a side
ACA_MAX_RANK_FRACTION = 1.0 / 3.0      # rank cap in element pivots, of the shorter side
ACA_CERTIFY_LINES = 3                  # exact element rows and columns of the certificate
ACA_CERTIFY_FACTOR = 3.0               # certificate limit, times the tolerance
ACA_RETRY_TOL_FACTOR = 10.0            # a failed certificate reruns the block at tol / this
ACA_SEED = 12345                       # seed of the sample and certificate lines
ACA_RECOMPRESS_MAX = 64                # recompress factors of at most this many columns (0: off)
COMPRESSED_NEAR_RADIUS_FACTOR = MIXED_NEAR_RADIUS_FACTOR   # FP64 closed form inside this radius
COMPRESSED_SCRATCH_BYTES = 4 << 30     # cross-approximation scratch per batch of blocks
COMPRESSED_VIEW_CACHE = 4              # material views kept per pair operator
