"""CPU restatement of the preconditioner network (test infrastructure only).

3-layer MLP 16 -> 128 -> 128 -> 2 with tanh, parameters packed as W1 [128][16],
b1 [128], W2 [128][128], b2 [128], W3 [2][128], b3 [2].  The forward pass uses
BF16-rounded parameters and rounds the inputs and hidden activations to BF16
(products accumulate in FP32); the backward pass is FP32 through the rounded
activations.  Used to check the GPU network kernels' outputs and gradients.
"""
import numpy as np

NF, NH, NO = 16, 128, 2
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NO * NH
NPARAM = OFF_B3 + NO


def bf16(x):
    """Round FP32 values to BF16 (round to nearest even) and back."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = 0x7FFF + ((u >> 16) & 1)
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(w):
    w = np.asarray(w, dtype=np.float32)
    return (w[OFF_W1:OFF_B1].reshape(NH, NF), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(NH, NH),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3].reshape(NO, NH), w[OFF_B3:NPARAM])


def forward(w, F):
    W1, b1, W2, b2, W3, b3 = [bf16(t) for t in unpack(w)]
    X = bf16(F)
    H1 = bf16(np.tanh(X.astype(np.float64) @ W1.T + b1).astype(np.float32))
    H2 = bf16(np.tanh(H1.astype(np.float64) @ W2.T + b2).astype(np.float32))
    O = (H2.astype(np.float64) @ W3.T + b3).astype(np.float32)
    return X, H1, H2, O


def backward(w, F, dO):
    W1, b1, W2, b2, W3, b3 = [bf16(t) for t in unpack(w)]
    X, H1, H2, O = forward(w, F)
    dO = np.asarray(dO, dtype=np.float64)
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = (dO.T @ H2).ravel()
    g[OFF_B3:NPARAM] = dO.sum(0)
    D2 = (dO @ W3) * (1.0 - H2.astype(np.float64) ** 2)
    g[OFF_W2:OFF_B2] = (D2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = D2.sum(0)
    D1 = (D2 @ W2) * (1.0 - H1.astype(np.float64) ** 2)
    g[OFF_W1:OFF_B1] = (D1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = D1.sum(0)
    return O, g
