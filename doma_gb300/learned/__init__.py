"""Learned source-iteration accelerator: the U-Net (net.py), its training
data (data.py) and training loop (train.py).  The network runs on the
library's own BF16 kernels through the doma_unet_* C ABI; PyTorch only holds
device buffers and assembles training batches."""
