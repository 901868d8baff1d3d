"""Thread-count helper of so3g.proj.mapthreads (python/proj/mapthreads.py:14-22).

The reference's dominant-scan-direction assignment (get_threads_domdir)
balances OpenMP threads over pixel-disjoint bands; the GPU kernels
accumulate with atomics and need no such bands, so Projectionist maps
method 'domdir' onto the 'simple' stripes.
"""


def get_num_threads(n_threads=None):
    if n_threads is None:
        import so3g_gb300
        return so3g_gb300.useful_info()['omp_num_threads']
    return n_threads
