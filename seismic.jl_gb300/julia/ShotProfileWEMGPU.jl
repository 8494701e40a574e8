# ShotProfileWEMGPU.jl -- batched GPU variant of Seismic.jl's ShotProfileWEM
# (src/Imaging/ShotProfileWEM.jl:39), in the package's Julia 0.6 dialect.
#
# The unmodified ShotProfileWEM already runs on the GPU once shotwem.so from this
# repository is first on LD_LIBRARY_PATH: it calls the library's `main` shot by shot
# (ShotProfileWEM.jl:334-349). This file adds the batched path: the whole survey goes
# to the GPU in one call (wem_prepare + wem_migrate / wem_model, include/shotwem_gb300.h)
# instead of one process per shot and file-based stacking (ShotProfileWEM.jl:100-199).
# Same keywords as ShotProfileWEM; nangx = nangy = 1 only.

const libshotwem = "shotwem"

immutable WemParams          # wem_params, field for field
    nt::Int32; ot::Float32; dt::Float32
    nmx::Int32; omx::Float32; dmx::Float32
    nmy::Int32; omy::Float32; dmy::Float32
    nz::Int32; oz::Float32; dz::Float32
    gz::Float32; sz::Float32
    nref::Int32; fmin::Float32; fmax::Float32
    padt::Int32; padx::Int32
    pspi::Int32; interp::Int32; precision::Int32; verbose::Int32
end

function wem_check(rc)
    if rc != 0
        msg = unsafe_string(ccall((:wem_last_error, libshotwem), Cstring, ()))
        error("shotwem status $rc: $msg")
    end
end

function ShotProfileWEMGPU(m::AbstractString, d::AbstractString, adj=true; pspi=true, nref=5, damping=1000.,
                           vel="vel", wav="wav", sz=0., gz=0., fmin=0, fmax=80, padt=2, padx=2,
                           verbose=false, sx=[0], sy=[0], interp="ref", device=0)
    v, hv, ev = SeisRead(vel)
    nx = hv[end].imx - hv[1].imx + 1
    ny = hv[end].imy - hv[1].imy + 1
    ox = hv[1].mx; dx = hv[2].mx - ox
    oy = hv[1].my; dy = ny > 1 ? hv[nx+1].my - oy : dx
    nz = hv[1].n1; dz = hv[1].d1; oz = hv[1].o1
    w, hw, ew = SeisRead(wav)
    nt = hw[1].n1; dt = hw[1].d1; ot = hw[1].o1
    p = WemParams(nt, ot, dt, nx, ox, dx, ny, oy, dy, nz, oz, dz, gz, sz, nref, fmin, fmax, padt, padx,
                  pspi ? 1 : 0, interp == "linear" ? 1 : 0, 0, verbose ? 1 : 0)
    sxv = convert(Array{Float32,1}, sx); syv = convert(Array{Float32,1}, sy)
    ctx = Ref{Ptr{Void}}(C_NULL)
    wem_check(ccall((:wem_ctx_create, libshotwem), Cint, (Ptr{Ptr{Void}}, Cint), ctx, device))
    try
        # v is (nz, nx*ny) column-major == C vel[ix][iz]
        wem_check(ccall((:wem_prepare, libshotwem), Cint, (Ptr{Void}, Ref{WemParams}, Ptr{Float32}, Ptr{Float32}),
                        ctx[], p, convert(Array{Float32,2}, v), convert(Array{Float32,1}, w[:, 1])))
        if adj
            dd, hd, ed = SeisRead(d)
            # traces of each shot (SeisWindow by sx, sy) and their grid cells from gx, gy
            off = Int64[0]; cells = Int32[]; cols = Int[]
            for i = 1 : length(sxv)
                for j = 1 : length(hd)
                    if hd[j].sx == sxv[i] && hd[j].sy == syv[i]
                        push!(cols, j)
                        ix = Int(round((hd[j].gx - ox)/dx)); iy = ny > 1 ? Int(round((hd[j].gy - oy)/dy)) : 0
                        push!(cells, Int32(ix*ny + iy))
                    end
                end
                push!(off, length(cols))
            end
            data = convert(Array{Float32,2}, dd[:, cols])        # (nt, ntrace)
            img = zeros(Float32, nz, nx*ny)
            wem_check(ccall((:wem_migrate, libshotwem), Cint,
                            (Ptr{Void}, Cint, Ptr{Float32}, Ptr{Float32}, Ptr{Int64}, Ptr{Int32}, Ptr{Float32}, Ptr{Float32}),
                            ctx[], length(sxv), sxv, syv, off, cells, data, img))
            h = Header[]
            for imx = 1 : nx, imy = 1 : ny
                hh = Seismic.InitSeisHeader()
                hh.tracenum = length(h) + 2; hh.o1 = 0; hh.n1 = nz; hh.d1 = dz
                hh.imx = imx - 1 + hv[1].imx; hh.imy = imy - 1 + hv[1].imy
                hh.mx = dx*hh.imx; hh.my = dy*hh.imy
                push!(h, hh)
            end
            extent = Seismic.Extent(nz, nx, ny, 1, 1, oz, ox, oy, 0, 0, dz, dx, dy, 1, 1,
                                    "Depth", "mx", "my", "angx", "angy", "m", "m", "m", "degrees", "degrees", "")
            SeisWrite(m, img, h, extent)
            return img
        else
            mm, hm, em = SeisRead(m)
            n = nx*ny
            off = Int64[n*(i-1) for i = 1 : length(sxv)+1]
            cells = Int32[j for i = 1 : length(sxv) for j = 0 : n-1]
            data = zeros(Float32, nt, n*length(sxv))
            wem_check(ccall((:wem_model, libshotwem), Cint,
                            (Ptr{Void}, Cint, Ptr{Float32}, Ptr{Float32}, Ptr{Int64}, Ptr{Int32}, Ptr{Float32}, Ptr{Float32}, Cint),
                            ctx[], length(sxv), sxv, syv, off, cells, convert(Array{Float32,2}, mm[:, 1:n]), data, 0))
            return data
        end
    finally
        ccall((:wem_ctx_destroy, libshotwem), Cint, (Ptr{Void},), ctx[])
    end
end
