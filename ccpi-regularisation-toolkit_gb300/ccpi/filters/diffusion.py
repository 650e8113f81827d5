"""Diffusion family: same functions and signatures as the reference's
src/Python/ccpi/filters/diffusion.py (NDF, Diff4th).

Non-linear diffusion runs deterministic Jacobi sweeps; the reference's C-OMP
sweep updates in place and depends on the thread count.
"""
from ._marshal import as_info, as_input, as_output, dims, ptr
from .utils import check_status, cilreg, cilregcuda


def NDF_CPU(inputData, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype, epsil, out=None, infovector=None):
    """Non-linear diffusion (Diffusion_core.c:53).  penaltytype: 1 Huber,
    2 Perona-Malik, 3 Tukey, 4 threshold-linear, 5 threshold-Huber; sigmaPar=0
    selects linear diffusion."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.Diffusion_CPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(sigmaPar),
                                   int(iterationsNumb), float(tau), int(penaltytype), float(epsil), *dims(a))
    check_status(st, cilreg)
    return out


def Diffus4th_CPU(inputData, lambdaPar, sigmaPar, iterationsNumb, tau, epsil, out=None, infovector=None):
    """Fourth-order anisotropic diffusion (Diffus4th_order_core.c:44)."""
    a = as_input(inputData)
    out = as_output(out, a)
    info = as_info(infovector)
    st = cilreg.Diffus4th_CPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(sigmaPar),
                                   int(iterationsNumb), float(tau), float(epsil), *dims(a))
    check_status(st, cilreg)
    return out


def _dev(gpu_device):
    return 0 if gpu_device == "gpu" else int(gpu_device)


def NDF_GPU(inputData, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype, epsil, gpu_device, out=None,
            infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.NonlDiff_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(sigmaPar),
                                      int(iterationsNumb), float(tau), int(penaltytype), float(epsil),
                                      _dev(gpu_device), *dims(a))
    check_status(st)
    return out


def Diffus4th_GPU(inputData, lambdaPar, sigmaPar, iterationsNumb, tau, epsil, gpu_device, out=None,
                  infovector=None):
    a = as_input(inputData)
    out = as_output(out, a, zero_init=int(iterationsNumb) <= 0)
    info = as_info(infovector)
    st = cilregcuda.Diffus4th_GPU_main(ptr(a), ptr(out), ptr(info), float(lambdaPar), float(sigmaPar),
                                       int(iterationsNumb), float(tau), float(epsil), _dev(gpu_device), *dims(a))
    check_status(st)
    return out
