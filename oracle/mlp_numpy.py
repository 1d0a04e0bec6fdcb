"""numpy restatement of the learned step-size proposer's MLP (forward and the
gradient of the mean squared error) -- the CPU checker of the GPU kernels in
instaheat_gb300/csrc/ih_mlp.cu.

TEST INFRASTRUCTURE ONLY.  The network has no reference counterpart; this is
the independent CPU computation its gradients are checked against.  It uses
the same BF16-rounded weights the kernels read (passed in as float32) and
evaluates in float64.
"""
import numpy as np

NI, NH = 12, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + NI * NH
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH
NP = OFF_B3 + 1
C_GELU = np.sqrt(2.0 / np.pi)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NI, NH), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3], p[OFF_B3])


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C_GELU * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    u = C_GELU * (x + 0.044715 * x ** 3)
    t = np.tanh(u)
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C_GELU * (1.0 + 3 * 0.044715 * x * x)


def forward(p, X, norm):
    mean, std, out_mean, out_std = norm
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = (np.asarray(X, np.float64) - mean) / std
    z1 = x @ W1 + b1
    h1 = gelu(z1)
    z2 = h1 @ W2 + b2
    h2 = gelu(z2)
    o = h2 @ W3 + b3
    return o * out_std + out_mean, (x, z1, h1, z2, h2, o)


def gradients(p, X, Y, norm):
    """d/dp of mean((o - (Y - out_mean)/out_std)^2); returns (grad[NP], loss)."""
    mean, std, out_mean, out_std = norm
    W1, b1, W2, b2, W3, b3 = unpack(p)
    _, (x, z1, h1, z2, h2, o) = forward(p, X, norm)
    t = (np.asarray(Y, np.float64) - out_mean) / out_std
    n = len(x)
    d = o - t
    loss = np.mean(d * d)
    dy = 2.0 * d / n
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = (dy[:, None] * W3[None, :]) * gelu_grad(z2)
    gW2 = h1.T @ dz2
    gb2 = dz2.sum(axis=0)
    dz1 = (dz2 @ W2.T) * gelu_grad(z1)
    gW1 = x.T @ dz1
    gb1 = dz1.sum(axis=0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return g, loss
