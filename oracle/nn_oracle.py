"""Oracle of the learned warm-start network (test infrastructure only): the
architecture of topopt.jl_gb300/csrc/tog_nn.cu restated with torch on the CPU
in float64, used to check the GPU forward pass and the gradients of the
GPU backward pass.  The network has no counterpart in TopOpt.jl.

Layout conventions shared with the library: tensors are channels-last
(batch, z, y, x, channels); the parameter vector holds, per layer,
W[cout][27][cin] (tap = 9 kz + 3 ky + kx) then b[cout]; input channels are
padded from 8 to 16 and the output from 3 to 16 channels."""
import numpy as np
import torch
import torch.nn.functional as F

LAYERS = [(16, 16, 1), (16, 32, 2), (32, 48, 2), (48, 64, 2), (64, 48, 1), (48, 32, 1), (32, 16, 1), (16, 16, 1)]


def n_params():
    return sum(27 * ci * co + co for ci, co, _ in LAYERS)


def unpack(params):
    """Parameter vector -> list of (weight [co, ci, 3, 3, 3], bias [co]) float64 tensors."""
    out, off = [], 0
    for ci, co, _ in LAYERS:
        w = torch.as_tensor(np.asarray(params[off:off + 27 * ci * co], dtype=np.float64)).reshape(co, 3, 3, 3, ci)
        off += 27 * ci * co
        b = torch.as_tensor(np.asarray(params[off:off + co], dtype=np.float64))
        off += co
        out.append((w.permute(0, 4, 1, 2, 3).contiguous().requires_grad_(True), b.clone().requires_grad_(True)))
    return out


def pack_grads(layers):
    parts = []
    for w, b in layers:
        parts.append(w.grad.permute(0, 2, 3, 4, 1).reshape(-1).numpy())
        parts.append(b.grad.numpy())
    return np.concatenate(parts)


def _up(x, like):
    """Nearest x2 upsampling: fine voxel (z, y, x) reads coarse (z // 2, y // 2, x // 2)."""
    d, h, w = like.shape[2:]
    iz, iy, ix = (torch.arange(n) // 2 for n in (d, h, w))
    return x[:, :, iz][:, :, :, iy][:, :, :, :, ix]


def forward(layers, inp):
    """inp: (batch, z, y, x, 8) array -> output (batch, z, y, x, 3) tensor."""
    x = torch.as_tensor(np.asarray(inp, dtype=np.float64)).permute(0, 4, 1, 2, 3)
    x = torch.cat([x, torch.zeros_like(x)], dim=1)

    def conv(l, t):
        w, b = layers[l]
        return F.conv3d(t, w, b, stride=LAYERS[l][2], padding=1)

    a0 = F.relu(conv(0, x))
    a1 = F.relu(conv(1, a0))
    a2 = F.relu(conv(2, a1))
    a3 = F.relu(conv(3, a2))
    b2 = F.relu(conv(4, _up(a3, a2)) + a2)
    b1 = F.relu(conv(5, _up(b2, a1)) + a1)
    b0 = F.relu(conv(6, _up(b1, a0)) + a0)
    y = conv(7, b0)
    return y[:, :3].permute(0, 2, 3, 4, 1)


def loss_and_grads(params, inp, target):
    """Mean squared error over batch x nodes x 3 and its gradient (parameter-vector layout)."""
    layers = unpack(params)
    y = forward(layers, inp)
    t = torch.as_tensor(np.asarray(target, dtype=np.float64))
    loss = ((y - t) ** 2).mean()
    loss.backward()
    return float(loss.detach()), pack_grads(layers)


def bf16_round(a):
    """Round to bfloat16 (nearest even) and back, as the GPU kernels read weights and inputs."""
    return torch.as_tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
