"""Device helpers with the reference's names (tedeous/device.py:7-52). The compute path needs a
CUDA device; solver_device only sets torch's default device as the reference does."""
import torch


def solver_device(device: str):
    if device in ('cuda', 'gpu') and torch.cuda.is_available():
        return torch.set_default_device('cuda')
    return torch.set_default_device('cpu')


def check_device(data):
    device = torch.tensor([0.]).device
    if isinstance(data, torch.Tensor):
        return data if data.device == device else data.to(device)
    return torch.tensor(data).to(device)


def device_type():
    return torch.tensor([0.]).device.type
