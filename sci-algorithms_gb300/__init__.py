"""GB300-native GAP-TV / ADMM-TV reconstruction for snapshot compressive imaging.

A drop-in for the TV path of Scientific-Research-Resource/SCI-algorithms
``PnP_SCI/python``: the ``A_`` / ``At_`` mask operators, the Chambolle TV
denoiser and the ``admmdenoise_cacti`` / ``gap_denoise`` / ``admm_denoise``
drivers, with the same names and arguments.  Compute runs in hand-written
sm_103a CUDA kernels behind the C ABI of ``include/sci_gb300.h``
(``libsci_gb300.so``); there is no CPU fallback.
"""
from .buildlib import build  # noqa: F401
from .utils import A_, At_, psnr, make_ops, MaskOperator  # noqa: F401
from .tv import (TVM, denoise_tv_chambolle, denoise_tv_matlab, tv_frames,  # noqa: F401
                 tv_matlab_frames)
from .pnp_sci_algo import (admmdenoise_cacti, gap_denoise, admm_denoise,  # noqa: F401
                           GAP_TV_rec, ADMM_TV_rec)
from .solver import Solver  # noqa: F401
from .bayer import gap_denoise_bayer, admm_denoise_bayer  # noqa: F401
from .joint import (joint_admmdenoise_cacti, gap_joint_denoise, admm_joint_denoise,  # noqa: F401
                    gap_multistep_denoise, admm_multistep_denoise)
from .cnn import (FFDNet, FastDVDnet, CnnEngine, ffdnet_vdenoiser,  # noqa: F401
                  fastdvdnet_denoiser, load_checkpoint, load_reference_state_dict,
                  reference_state_dict)
from .cassi import CassiOperator, CassiSolver, make_cassi_ops  # noqa: F401
from .unrolled import (UnrolledGapTV, unrolled_loss, unrolled_workspace,  # noqa: F401
                       torch_unrolled_loss)
from .batch import BatchSolver  # noqa: F401
from . import datasets  # noqa: F401
