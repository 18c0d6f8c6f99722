"""Distorted camera captures of painted symbols, rendered on the GPU with torch (test and benchmark tooling; the
library never imports it).

A page is the sender's grey page (the library's GPU encoder, lizg_encode_dev: the reference's lizard_encode +
lizard_paint_grey within one grey level, the picture's cyclic guard and the border included) seen through a camera:
a view H (layout modules -> ideal image pixels), radial distortion k1 about the frame centre (r over the
half-diagonal), a Gaussian blur of sigma pixels in linear light (grey -> (g / 255)^gamma -> blur -> ^(1 / gamma)),
AWGN, 8 bits. The same model as synth.distorted_capture, which renders in numpy on the host; this one renders a
batch of frames on the device in a fraction of the time, and takes the page with its border and guard."""
import numpy as np

from . import synth

QUIET = 2   # the page's quiet margin, modules a side


class _Fmt:
    def __init__(self, n, span):
        self.n, self.span = n, span


def views(n, span, width, height, seeds, base_side):
    """A distorted_view a seed: rotation U(+-15 deg), tilt U(+-20 deg), the layout's side base_side x U(0.8, 1.1)."""
    return [synth.distorted_view(_Fmt(n, span), width, height, np.random.default_rng(s), base_side=base_side) for s in seeds]


def corner_homography(span, H, k1, width, height):
    """What a finder's corners give: the homography through the layout's four corners as the camera sees them."""
    side = span + 30
    corners = np.array([[0, 0], [side, 0], [side, side], [0, side]], np.float64)
    q = np.asarray(H, np.float64).reshape(3, 3) @ np.column_stack([corners, np.ones(4)]).T
    cu, cv = synth.radial(q[0] / q[2], q[1] / q[2], width, height, k1)
    return synth.homography_4(corners, np.column_stack([cu, cv]))


def registration(span, H, k1, width, height, true_mesh=False):
    """The registration the receiver takes (H, then the node mesh): the corners' homography with a zero mesh, or with
    true_mesh the mesh of the camera's true displacements about it at every node (the best a registration can be)."""
    Hp = corner_homography(span, H, k1, width, height)
    nx = synth.layout_nodes(span)
    if not true_mesh:
        return np.concatenate([Hp.astype(np.float32), np.zeros(2 * nx.size * nx.size, np.float32)])
    X, Y = np.meshgrid(nx, nx)
    pts = np.stack([X.ravel(), Y.ravel(), np.ones(X.size)])
    q = np.asarray(H, np.float64).reshape(3, 3) @ pts
    tu, tv = synth.radial(q[0] / q[2], q[1] / q[2], width, height, k1)
    p = Hp.reshape(3, 3) @ pts
    d = np.stack([tu - p[0] / p[2], tv - p[1] / p[2]], 1).astype(np.float32)
    return np.concatenate([Hp.astype(np.float32), d.ravel()])


def _blur(img, sigma, torch):
    """Separable Gaussian of sigma pixels, the edges held (scipy.ndimage's 'nearest')."""
    r = max(1, int(4.0 * sigma + 0.5))
    x = torch.arange(-r, r + 1, dtype=img.dtype, device=img.device)
    k = torch.exp(-0.5 * (x / sigma) ** 2)
    k = k / k.sum()
    im = img[None, None]
    im = torch.nn.functional.pad(im, (r, r, 0, 0), mode="replicate")
    im = torch.nn.functional.conv2d(im, k.view(1, 1, 1, -1))
    im = torch.nn.functional.pad(im, (0, 0, r, r), mode="replicate")
    im = torch.nn.functional.conv2d(im, k.view(1, 1, -1, 1))
    return im[0, 0]


def capture(page, pxm, width, height, H, k1, blur, sigma, seed, mid=128.0, gamma=2.2):
    """One capture (height x width uint8 on the page's device) of a grey page (W x W uint8 torch tensor, quiet margin
    included) through view H, radial k1, blur in linear light, AWGN of sigma grey levels (a generator seeded by seed)."""
    import torch
    dev = page.device
    Wp = page.shape[0]
    Hi = torch.tensor(np.linalg.inv(np.asarray(H, np.float64).reshape(3, 3)), dtype=torch.float64, device=dev)
    V, U = torch.meshgrid(torch.arange(height, dtype=torch.float64, device=dev) + 0.5, torch.arange(width, dtype=torch.float64, device=dev) + 0.5,
                          indexing="ij")
    cx, cy, R = width / 2.0, height / 2.0, float(np.hypot(width, height)) / 2.0
    u, v = U.clone(), V.clone()
    for _ in range(8):   # the inverse of the radial map by fixed-point rounds
        dx, dy = u - cx, v - cy
        g = 1 + k1 * (dx * dx + dy * dy) / (R * R)
        u, v = cx + (U - cx) / g, cy + (V - cy) / g
    qw = Hi[2, 0] * u + Hi[2, 1] * v + Hi[2, 2]
    mx = (Hi[0, 0] * u + Hi[0, 1] * v + Hi[0, 2]) / qw
    my = (Hi[1, 0] * u + Hi[1, 1] * v + Hi[1, 2]) / qw
    sx, sy = (mx + QUIET) * pxm - 0.5, (my + QUIET) * pxm - 0.5
    inside = (sx >= 0) & (sy >= 0) & (sx <= Wp - 1.001) & (sy <= Wp - 1.001)
    x0 = torch.clamp(torch.floor(sx), 0, Wp - 2).long()
    y0 = torch.clamp(torch.floor(sy), 0, Wp - 2).long()
    fx, fy = torch.clamp(sx - x0, 0, 1), torch.clamp(sy - y0, 0, 1)
    p = page.to(torch.float64)
    val = (p[y0, x0] * (1 - fx) + p[y0, x0 + 1] * fx) * (1 - fy) + (p[y0 + 1, x0] * (1 - fx) + p[y0 + 1, x0 + 1] * fx) * fy
    img = torch.where(inside, val, torch.full_like(val, mid))
    if blur > 0:
        img = 255.0 * torch.clamp(_blur((img / 255.0) ** gamma, blur, torch), 0, 1) ** (1.0 / gamma)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    noise = torch.randn(img.shape, generator=gen, device=dev, dtype=torch.float64)
    return torch.clamp(torch.round(img + sigma * noise), 0, 255).to(torch.uint8)


def pages(lz, n, subch, span, block_rows, pilots, chunk=64):
    """The sender's grey pages of frames of blocks (frames x blocks x 476 uint8), painted on the GPU: a torch tensor
    frames x W x W, and the page's pixels a module."""
    import ctypes
    import torch
    enc = lz.Encoder(n, subch, span, max_frames=chunk)
    frames = block_rows.shape[0]
    out = torch.empty((frames, enc.W, enc.W), dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    for a in range(0, frames, chunk):
        b = torch.from_numpy(np.ascontiguousarray(block_rows[a:a + chunk])).cuda()
        k = b.shape[0]
        lz._check(lz.lib().lizg_encode_dev(enc._h, ctypes.c_void_p(b.data_ptr()), k, int(pilots[a]) if np.ndim(pilots) else int(pilots), None,
                                           ctypes.c_void_p(out[a:a + k].data_ptr()), ctypes.c_void_p(st)), "lizg_encode_dev")
    torch.cuda.synchronize()
    return out, enc.pxm
