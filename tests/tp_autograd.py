"""torch.autograd.Function over the binned Gaussian log-likelihood: forward
runs the GPU forward pass, backward the GPU adjoint pass (test harness)."""
import torch


class LogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, model):
        t = theta.detach().cpu().double().tolist()
        lnl, grad, _, _ = model.gradient(t)  # forward + adjoint on the device
        ctx.save_for_backward(torch.tensor(grad, dtype=theta.dtype))
        return torch.tensor(lnl, dtype=theta.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return grad_out * grad, None


def log_likelihood(theta, model):
    return LogLikelihood.apply(theta, model)
