# ShotProfileWEMGPU.jl -- batched GPU variant of Seismic.jl's ShotProfileWEM
# (src/Imaging/ShotProfileWEM.jl:39), in the package's Julia 0.6 dialect.
#
# The unmodified ShotProfileWEM already runs on the GPU once shotwem.so from this
# repository is first on LD_LIBRARY_PATH: it calls the library's `main` shot by shot
# (ShotProfileWEM.jl:334-349). This file adds the batched path: the whole survey goes
# to the GPU in one call (wem_prepare + wem_migrate / wem_model, include/shotwem_gb300.h)
# instead of one process per shot and file-based stacking (ShotProfileWEM.jl:100-199).
# Same keywords as ShotProfileWEM, angle gathers (nangx, nangy > 1) included: each shot's
# image is binned by that shot's incidence angles (files written by ComputeAngles), and
# demigration unbins the gathers at each shot's own angles (ShotProfileWEM.jl:155-188,
# 228-270). The Python mirror seismic.jl_gb300/wemgpu/shotprofile.py is the tested one.

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

function wem_migrate_shots(ctx, sxv, syv, off, cells, data, nz, n)
    img = zeros(Float32, nz, n)
    wem_check(ccall((:wem_migrate, libshotwem), Cint,
                    (Ptr{Void}, Cint, Ptr{Float32}, Ptr{Float32}, Ptr{Int64}, Ptr{Int32}, Ptr{Float32}, Ptr{Float32}),
                    ctx, length(sxv), sxv, syv, off, cells, data, img))
    return img
end

function wem_model_shots(ctx, sxv, syv, img, nt, n)
    off = Int64[n*(i-1) for i = 1 : length(sxv)+1]
    cells = Int32[j for i = 1 : length(sxv) for j = 0 : n-1]
    data = zeros(Float32, nt, n*length(sxv))
    wem_check(ccall((:wem_model, libshotwem), Cint,
                    (Ptr{Void}, Cint, Ptr{Float32}, Ptr{Float32}, Ptr{Int64}, Ptr{Int32}, Ptr{Float32}, Ptr{Float32}, Cint),
                    ctx, length(sxv), sxv, syv, off, cells, convert(Array{Float32,2}, img), data, 0))
    return data
end

# The traces of the shots (SeisWindow by sx, sy: ShotProfileWEM.jl:101-103) in compact form,
# placed on the grid by their receiver positions gx, gy.
function window_shots(dd, hd, sxv, syv, ox, dx, oy, dy, nx, ny)
    off = Int64[0]; cells = Int32[]; cols = Int[]
    for i = 1 : length(sxv)
        for j = 1 : length(hd)
            if hd[j].sx == sxv[i] && hd[j].sy == syv[i]
                ix = Int(round((hd[j].gx - ox)/dx)); iy = ny > 1 ? Int(round((hd[j].gy - oy)/dy)) : 0
                if ix >= 0 && ix < nx && iy >= 0 && iy < ny
                    push!(cols, j)
                    push!(cells, Int32(ix*ny + iy))
                end
            end
        end
        push!(off, length(cols))
    end
    return off, cells, convert(Array{Float32,2}, dd[:, cols])    # (nt, ntrace)
end

# The section of the shot at (x0, y0) in an angle file written by ComputeAngles
# (ShotProfileWEM.jl:93-97), (nz, n).
function shot_angles(name, x0, y0, n)
    a, h, e = SeisRead(name)
    sel = Int[j for j = 1 : length(h) if h[j].sx == x0 && h[j].sy == y0]
    length(sel) == n || error("$name: $(length(sel)) traces for the shot at sx=$x0, sy=$y0, need $n")
    return convert(Array{Float64,2}, a[:, sel])
end

# The bilinear bins of one sample's angles (ShotProfileWEM.jl:161-176): (weight, bin) of each
# term that applies, bins 1-based with angy fastest. The fourth term's guard is iangx < nangx,
# the forward side's (:264-266); the adjoint side's `iang < nang` (:183) names no variable.
function angle_terms(ax, ay, nangx, oangx, dangx, nangy, oangy, dangy)
    iangx = Int(floor((ax - oangx)/dangx)) + 1
    angx1 = (iangx - 1)*dangx + oangx; angx2 = angx1 + dangx
    iangy = Int(floor((ay - oangy)/dangy)) + 1
    angy1 = (iangy - 1)*dangy + oangy; angy2 = angy1 + dangy
    den = (angx2 - angx1)*(angy2 - angy1)
    terms = Tuple{Float64,Int}[]
    if iangx >= 1 && iangx <= nangx && iangy >= 1 && iangy <= nangy
        b1 = (iangx - 1)*nangy + iangy
        push!(terms, ((angx2 - ax)*(angy2 - ay)/den, b1))
        if iangx < nangx
            push!(terms, ((ax - angx1)*(angy2 - ay)/den, b1 + nangy))
        end
        if nangy > 1
            push!(terms, ((angx2 - ax)*(ay - angy1)/den, b1 + 1))
            if iangx < nangx
                push!(terms, ((ax - angx1)*(ay - angy1)/den, b1 + nangy + 1))
            end
        end
    end
    return terms
end

function ShotProfileWEMGPU(m::AbstractString, d::AbstractString, adj=true; pspi=true, nref=5, damping=1000.,
                           vel="vel", angx="angx", angy="angy", wav="wav", sz=0., gz=0.,
                           nangx=1, oangx=0, dangx=1, nangy=1, oangy=0, dangy=1, fmin=0, fmax=80, padt=2,
                           padx=2, verbose=false, sx=[0], sy=[0], interp="ref", device=0)
    v, hv, ev = SeisRead(vel)
    nx = hv[end].imx - hv[1].imx + 1
    ny = hv[end].imy - hv[1].imy + 1
    ox = hv[1].mx; dx = hv[2].mx - ox
    oy = hv[1].my; dy = ny > 1 ? hv[nx+1].my - oy : dx
    nz = hv[1].n1; dz = hv[1].d1; oz = hv[1].o1
    n = nx*ny
    w, hw, ew = SeisRead(wav)
    nt = hw[1].n1; dt = hw[1].d1; ot = hw[1].o1
    p = WemParams(nt, ot, dt, nx, ox, dx, ny, oy, dy, nz, oz, dz, gz, sz, nref, fmin, fmax, padt, padx,
                  pspi ? 1 : 0, interp == "linear" ? 1 : 0, 0, verbose ? 1 : 0)
    sxv = convert(Array{Float32,1}, sx); syv = convert(Array{Float32,1}, sy)
    if length(syv) == 1 && length(sxv) > 1
        syv = fill(syv[1], length(sxv))
    end
    gathers = nangx != 1 || nangy != 1
    nang = nangx*nangy
    ctx = Ref{Ptr{Void}}(C_NULL)
    wem_check(ccall((:wem_ctx_create, libshotwem), Cint, (Ptr{Ptr{Void}}, Cint), ctx, device))
    try
        # v is (nz, nx*ny) column-major == C vel[ix][iz]
        wem_check(ccall((:wem_prepare, libshotwem), Cint, (Ptr{Void}, Ref{WemParams}, Ptr{Float32}, Ptr{Float32}),
                        ctx[], p, convert(Array{Float32,2}, v), convert(Array{Float32,1}, w[:, 1])))
        if adj
            dd, hd, ed = SeisRead(d)
            if gathers
                # every shot's image binned by its own incidence angles (ShotProfileWEM.jl:155-188)
                out = zeros(Float64, nz, nang, n)
                for i = 1 : length(sxv)
                    off, cells, data = window_shots(dd, hd, sxv[i:i], syv[i:i], ox, dx, oy, dy, nx, ny)
                    img = wem_migrate_shots(ctx[], sxv[i:i], syv[i:i], off, cells, data, nz, n)
                    ax = shot_angles(angx, sxv[i], syv[i], n); ay = shot_angles(angy, sxv[i], syv[i], n)
                    for ix = 1 : n, iz = 1 : nz
                        for (wt, b) in angle_terms(ax[iz, ix], ay[iz, ix], nangx, oangx, dangx, nangy, oangy, dangy)
                            out[iz, b, ix] += wt*img[iz, ix]
                        end
                    end
                end
                img = convert(Array{Float32,2}, reshape(out, nz, nang*n))
            else
                off, cells, data = window_shots(dd, hd, sxv, syv, ox, dx, oy, dy, nx, ny)
                img = wem_migrate_shots(ctx[], sxv, syv, off, cells, data, nz, n)
            end
            # image headers (ShotProfileWEM.jl:115-137): one trace per (imx, imy, iangx, iangy)
            h = Header[]
            for imx = 1 : nx, imy = 1 : ny, ia = 1 : nangx, iaz = 1 : nangy
                hh = Seismic.InitSeisHeader()
                hh.tracenum = length(h) + 2; hh.o1 = 0; hh.n1 = nz; hh.d1 = dz
                hh.imx = imx - 1 + hv[1].imx; hh.imy = imy - 1 + hv[1].imy
                hh.mx = dx*hh.imx; hh.my = dy*hh.imy
                hh.iang = ia - 1; hh.ang = (ia - 1)*dangx + oangx
                hh.iaz = iaz - 1; hh.az = (iaz - 1)*dangy + oangy
                push!(h, hh)
            end
            extent = Seismic.Extent(nz, nx, ny, nangx, nangy, oz, ox, oy, oangx, oangy, dz, dx, dy, dangx, dangy,
                                    "Depth", "mx", "my", "angx", "angy", "m", "m", "m", "degrees", "degrees", "")
            SeisWrite(m, img, h, extent)
            return img
        else
            mm, hm, em = SeisRead(m)
            if gathers
                # each shot sees the gathers at its own incidence angles (ShotProfileWEM.jl:228-270)
                gath = reshape(convert(Array{Float64,2}, mm[:, 1:nang*n]), nz, nang, n)
                data = zeros(Float32, nt, 0)
                for i = 1 : length(sxv)
                    ax = shot_angles(angx, sxv[i], syv[i], n); ay = shot_angles(angy, sxv[i], syv[i], n)
                    img = zeros(Float64, nz, n)
                    for ix = 1 : n, iz = 1 : nz
                        for (wt, b) in angle_terms(ax[iz, ix], ay[iz, ix], nangx, oangx, dangx, nangy, oangy, dangy)
                            img[iz, ix] += wt*gath[iz, b, ix]
                        end
                    end
                    data = hcat(data, wem_model_shots(ctx[], sxv[i:i], syv[i:i], img, nt, n))
                end
            else
                data = wem_model_shots(ctx[], sxv, syv, mm[:, 1:n], nt, n)
            end
            # every shot recorded on every grid cell, keyed by sx, sy (ShotProfileWEM.jl:210-309)
            h = Header[]
            for i = 1 : length(sxv), imx = 1 : nx, imy = 1 : ny
                hh = Seismic.InitSeisHeader()
                hh.tracenum = length(h) + 1; hh.n1 = nt; hh.d1 = dt; hh.o1 = ot
                hh.sx = sxv[i]; hh.sy = syv[i]
                hh.gx = ox + dx*(imx - 1); hh.gy = oy + dy*(imy - 1)
                hh.mx = hh.gx; hh.my = hh.gy; hh.hx = hh.gx - hh.sx; hh.hy = hh.gy - hh.sy
                hh.imx = imx - 1; hh.imy = imy - 1
                push!(h, hh)
            end
            nsx = length(sxv)
            extent = Seismic.Extent(nt, nx, ny, nsx, 1, ot, ox, oy, sxv[1], syv[1], dt, dx, dy,
                                    nsx > 1 ? sxv[2] - sxv[1] : 1, 1,
                                    "Time", "gx", "gy", "sx", "sy", "s", "m", "m", "m", "m", "")
            SeisWrite(d, data, h, extent)
            return data
        end
    finally
        ccall((:wem_ctx_destroy, libshotwem), Cint, (Ptr{Void},), ctx[])
    end
end
