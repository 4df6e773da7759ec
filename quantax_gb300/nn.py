"""Final activations of the ResConv model (quantax/nn/activation.py:7-32).

ResConv(final_activation=...) takes one of these two functions: the kernels implement them
inside the forward pass, so the functions here only name the choice and evaluate the same
mathematics on a host or device tensor (psi per final feature, before the mean over sites and
channels)."""
import torch


def exp_by_scale(x: torch.Tensor) -> torch.Tensor:
    """f(x) = exp(x) (the default)."""
    return torch.exp(x)


def sinhp1_by_scale(x: torch.Tensor) -> torch.Tensor:
    """f(x) = sinh(x) + 1."""
    return torch.sinh(x) + 1
