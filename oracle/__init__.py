"""CPU oracle for the GAP/ADMM-TV path (test infrastructure only; see the
module docstrings of ``reference_port`` and ``tv_chambolle``)."""
