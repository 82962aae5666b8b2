"""One representative launch sequence per kernel family, for ncu captures.

    python -m matrixmultiplicationcuda_gb300.profile_kernels [--only NAME,...] [--launches 3]

Families (seeded synthetic inputs; a few hundred MB on the device at most):
  tc        k_bcsr_tc: A 16384^2, 64x16 blocks, random 2 %, N 512, fp16, a
            512-column tile with one accumulator, static item stride
  plan_c3   k_bcsr_tc on a per-matrix plan: the same product in bf16 with the
            default tcgen05 configuration (256-column tile, five-group ring,
            two accumulators), items heaviest first from the plan's queue
  plan_c3_512  the same product in fp16 on a plan with a 512-column tile and
            one accumulator (one item per CTA), each launch started with
            SPMM_RUN_INPUTS_READY after the first
  tc_split  k_bcsr_tc in split fp16 (three MMAs per block), same product
  mma_e4m3  k_bcsr_mma: the same product in e4m3 with per-block scales
  mma16     k_bcsr_mma: A 8192^2, 16x16 blocks, random 5 %, N 1024, fp16
  batch     k_bcsr_tc_batch: the 64-product uneven workload, one launch
  convert   k_dense_to_bcsr (count and fill) + k_scan_counts: dense fp16
            8192 x 8192 (134 MB) with 16x16 blocks at 5 %
  quantize  k_to_f16 / k_to_bf16 / k_absmax / k_to_e4m3: 64 M fp32 values
  mlp       the cost model's forward / backward / AdamW kernels, batch 2000
  hybrid    k_bcsr_tc with the CSR pass in its epilogue (spmm_hcsr_mm): A 4096^2
            (10 % dense 16x16 blocks + 2 % scattered entries), threshold 0.5,
            N 1024
  hybrid_plan  the same product planned: CSR entries as gather blocks
  csr       k_csr_mm on the same matrix's entries, all as CSR
  tc64      k_bcsr_tc64 (64-row blocks, M=64 UMMAs, one CTA per SM): the tc
            product in fp16 and in split fp16, 256-column tile
  plan      k_bcsr_tc on a per-matrix plan: A 8192^2, 64x16 blocks, log-normal
            rows (5 %, CV 1.5), N 512, bf16, 256-column tile (rows far above
            the average load split into parts)
  dense     k_dense_tc: the native dense comparator, A 8192 x 8192, B 8192 x 1024, fp16
  gen       the GPU generators: k_gen_structure + k_gen_values for the tc
            product's structure (A 16384^2, 64x16, 2 %), k_gen_dense for B
            (16384 x 512), k_gen_matrix (reference blockrandom, 8192^2 fp16)
Each family runs `--launches` times after one warm-up, then synchronises and
checks the device error word.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="tc,tc_split,mma_e4m3,mma16,batch,convert,quantize,mlp,hybrid,hybrid_plan,csr,"
                                      "tc64,gen,dense,plan,plan_c3,plan_c3_512")
    ap.add_argument("--launches", type=int, default=3)
    args = ap.parse_args(argv)
    import torch
    import matrixmultiplicationcuda_gb300 as m
    from matrixmultiplicationcuda_gb300 import costmodel
    dev = torch.device("cuda", 0)
    only = set(args.only.split(","))
    L = args.launches

    def c3(dtype):
        M = K = 16384
        N = 512
        rp, ci = m.gen_structure(M, K, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240)
        vals = m.gen_values(len(ci), 64, 16, m.DIST_SCALED_NORMAL, seed=20241)
        Bf = m.gen_dense(K, N, m.DIST_NORMAL, seed=20242)
        A = m.BCSR.from_host(M, K, 64, rp, ci, vals, dtype, device=dev)
        Bq, Blo, Bs = m.quantize(torch.from_numpy(Bf).to(dev).reshape(-1), dtype)
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        return A, Bq.view(K, N), (Blo.view(K, N) if Blo is not None else None), \
            (float(Bs[0]) if Bs is not None else 1.0), C

    def run(fn):
        fn()
        torch.cuda.synchronize()
        for _ in range(L):
            fn()
        torch.cuda.synchronize()
        m.device_error_check()

    if "tc" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        cfg = m.Config(kernel=2, n_tile=512, acc_buffers=1)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg))
        print("tc: nnzb=%d" % A.nnzb)
    if "tc_split" in only:
        A, B, Blo, bs, C = c3(m.DType.F16_SPLIT)
        cfg = m.Config(kernel=2, n_tile=256, acc_buffers=2, stages=2)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg, B_lo=Blo))
        print("tc_split: nnzb=%d" % A.nnzb)
    if "mma_e4m3" in only:
        A, B, Blo, bs, C = c3(m.DType.E4M3)
        cfg = m.Config(kernel=1, n_tile=128, stages=4)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=cfg, b_scale=bs))
        print("mma_e4m3: nnzb=%d" % A.nnzb)
    if "mma16" in only:
        M = K = 8192
        N = 1024
        rp, ci = m.gen_structure(M, K, 16, m.PATTERN_RANDOM, 0.05, 0, seed=7)
        vals = m.gen_values(len(ci), 16, 16, m.DIST_UNIFORM, seed=8)
        A = m.BCSR.from_host(M, K, 16, rp, ci, vals, m.DType.F16, device=dev)
        B = torch.from_numpy(m.gen_dense(K, N, m.DIST_UNIFORM, seed=9)).to(dev).half()
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        cfg = m.Config(kernel=1, n_tile=256, stages=4)
        run(lambda: m.spmm(A, B, N=N, C=C, cfg=cfg))
        print("mma16: nnzb=%d" % A.nnzb)
    if "batch" in only:
        probs = []
        for sp in m.uneven_batch_specs(64, seed=2024):
            rp, ci, vals, Bf = m.make_problem(sp)
            A = m.BCSR.from_host(sp["M"], sp["K"], sp["bR"], rp, ci, vals, m.DType.F16, device=dev)
            probs.append((A, torch.from_numpy(Bf).to(dev).half(),
                          torch.empty((sp["M"], sp["N"]), dtype=torch.float32, device=dev)))
        plan = m.BatchPlan(probs)
        run(plan.run)
        plan.close()
        print("batch: %d problems" % len(probs))
    if "convert" in only:
        M = K = 8192
        rp, ci = m.gen_structure(M, K, 16, m.PATTERN_RANDOM, 0.05, 0, seed=11)
        vals = m.gen_values(len(ci), 16, 16, m.DIST_UNIFORM, seed=12)
        dense = torch.zeros((M, K), dtype=torch.float16, device=dev)
        blocks = torch.from_numpy(vals.reshape(-1, 16, 16)).to(dev).half()
        rows = np.repeat(np.arange(M // 16), np.diff(rp))
        view = dense.view(M // 16, 16, K // 16, 16).permute(0, 2, 1, 3)
        view[torch.from_numpy(rows).to(dev), torch.from_numpy(ci.astype(np.int64)).to(dev)] = blocks
        run(lambda: m.dense_to_bcsr(dense, 16, 16))
        print("convert: %d x %d, nnzb=%d" % (M, K, len(ci)))
    if "quantize" in only:
        src = torch.randn(64 << 20, device=dev) * 10
        for dt in (m.DType.F16, m.DType.BF16, m.DType.E4M3):
            run(lambda: m.quantize(src, dt, block_elems=1024))
        print("quantize: %d values" % src.numel())
    if only & {"hybrid", "hybrid_plan", "csr"}:
        M = K = 4096
        N = 1024
        blocks = m.generate_matrix(M, K, 0.9, "blockrandom", 16, seed=7)
        scatter = m.generate_matrix(M, K, 0.98, "random", 16, seed=8)
        A = np.where(blocks != 0, blocks, scatter).astype(np.float16).view(np.uint16)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        B = t(m.gen_dense(K, N, m.DIST_UNIFORM, seed=9)).half()
        C = torch.empty((M, N), dtype=torch.float32, device=dev)
        (bh, bi, bd), (ch, cx, cd) = m.host_dense_to_hcsr(A, 0.5)
        Ab = m.BCSR(M, K, 16, 16, t(bh), t(bi), t(bd.view(np.float16)))
        if "hybrid" in only:
            run(lambda: m.hcsr_mm(Ab, t(ch), t(cx), t(cd.view(np.float16)), B, N=N, C=C))
            print("hybrid: %d blocks, %d CSR entries" % (len(bi), len(cx)))
        if "hybrid_plan" in only:
            plan = m.HcsrPlan(Ab, t(ch), t(cx), t(cd.view(np.float16)))
            run(lambda: plan.run(B, N=N, C=C))
            print("hybrid_plan: (blocks, gather blocks) =", plan.info())
            plan.close()
        if "csr" in only:
            _, (rh, rx, rd) = m.host_dense_to_hcsr(A, 1.1)
            rh, rx, rd = t(rh), t(rx), t(rd.view(np.float16))
            run(lambda: m.csr_mm(rh, rx, rd, K, B, N=N, C=C))
            print("csr: %d entries" % rx.numel())
    if "plan_c3" in only:
        A, B, Blo, bs, C = c3(m.DType.BF16)
        plan = m.BcsrPlan(A, 512)
        run(lambda: plan.run(A, B, C=C))
        print("plan_c3: nnzb=%d, (items, split rows) = %s" % (A.nnzb, plan.info()[:2]))
        plan.close()
    if "plan_c3_512" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        plan = m.BcsrPlan(A, 512, m.Config(kernel=2, n_tile=512, acc_buffers=1))
        torch.cuda.synchronize()   # no kernel after this writes A or B
        run(lambda: plan.run(A, B, C=C, inputs_ready=True))
        print("plan_c3_512: nnzb=%d, (items, split rows) = %s" % (A.nnzb, plan.info()[:2]))
        plan.close()
    if "tc64" in only:
        A, B, Blo, bs, C = c3(m.DType.F16)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=m.Config(kernel=3, n_tile=256)))
        A, B, Blo, bs, C = c3(m.DType.F16_SPLIT)
        run(lambda: m.spmm(A, B, N=512, C=C, cfg=m.Config(kernel=3, n_tile=256), B_lo=Blo))
        print("tc64: nnzb=%d" % A.nnzb)
    if "plan" in only:
        M = K = 8192
        rp, ci = m.gen_structure(M, K, 64, m.PATTERN_LOGNORMAL, 0.05, 1.5, seed=77)
        vals = m.gen_values(len(ci), 64, 16, m.DIST_UNIFORM, seed=1)
        A = m.BCSR.from_host(M, K, 64, rp, ci, vals, m.DType.BF16, device=dev)
        B = torch.from_numpy(m.gen_dense(K, 512, m.DIST_UNIFORM, seed=2)).to(dev).bfloat16()
        C = torch.empty((M, 512), dtype=torch.float32, device=dev)
        plan = m.BcsrPlan(A, 512, m.Config(kernel=2, n_tile=256, acc_buffers=2))
        run(lambda: plan.run(A, B, C=C))
        print("plan: (items, split rows) =", plan.info()[:2])
        plan.close()
    if "dense" in only:
        g = torch.Generator().manual_seed(0)
        Ad = (torch.rand((8192, 8192), generator=g) * 2 - 1).half().to(dev)
        Bd = (torch.rand((8192, 1024), generator=g) * 2 - 1).half().to(dev)
        Cd = torch.empty((8192, 1024), dtype=torch.float32, device=dev)
        run(lambda: m.dense_mm(Ad, Bd, C=Cd))
        print("dense: 8192 x 8192 x 1024")
    if "gen" in only:
        def gen():
            rp, ci = m.gpu_gen_structure(16384, 16384, 64, m.PATTERN_RANDOM, 0.02, 0, seed=20240, device=dev)
            m.gpu_gen_values(ci.numel(), 64, 16, m.DIST_SCALED_NORMAL, seed=20241, device=dev)
            m.gpu_gen_dense(16384, 512, m.DIST_NORMAL, seed=20242, device=dev)
            m.gpu_generate_matrix(8192, 8192, 0.9, "blockrandom", 16, seed=7, device=dev)
        run(gen)
        print("gen: done")
    if "mlp" in only:
        s = costmodel.shape()
        rng = np.random.default_rng(0)
        p = costmodel.init_params(s, np.zeros(s.in_, np.float32), np.ones(s.in_, np.float32))
        net = costmodel.MLP(s, p, device=dev)
        X = torch.from_numpy(rng.standard_normal((2000, s.in_)).astype(np.float32)).to(dev)
        T = torch.from_numpy(rng.standard_normal((2000, s.out)).astype(np.float32)).to(dev)
        Mk = torch.ones_like(T)
        run(lambda: net.forward(X))
        run(lambda: net.loss_grad(X, T, Mk))
        print("mlp: batch 2000")


if __name__ == "__main__":
    main()
