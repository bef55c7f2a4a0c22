// The compute section of the reference's Renderer.draw (Astro/Renderer.swift:
// 505-542) on libastro_cuda: the Metal encoders for generateMortonCodes, the
// radix sort, the layered build, barnesHut and updateSpheres become calls into
// the C ABI. Buffers keep the reference's PositionMass / VelocityRadius /
// ColorType layouts (bridge.h), so the arrays built by makeSpheres are passed
// as they are.
import CAstroCUDA

public enum AstroError: Error {
    case status(Int32, String)
}

public final class AstroStep {
    private var ctx: OpaquePointer?

    /// Renderer.makeBuffers (Renderer.swift:336-391): one context for up to
    /// `maxCount` particles. `reference` selects the reference's constants.
    public init(maxCount: UInt32, reference: Bool = true) throws {
        var p = astro_params()
        try check(astro_params_default(reference ? 0 : 1, &p))
        var c: OpaquePointer?
        try check(astro_create(&p, maxCount, 1, &c))
        ctx = c
    }

    deinit { if let c = ctx { _ = astro_destroy(c) } }

    /// makeSpheres' buffer copy (Renderer.swift:490-492); the first
    /// `treeCount` particles go into the octree (octreeCount, :36).
    public func upload(_ positions: [PositionMass], _ velocities: [VelocityRadius],
                       _ colors: [ColorType], treeCount: UInt32) throws {
        try check(astro_upload(ctx, positions, velocities, colors,
                               UInt32(positions.count), treeCount))
    }

    /// One frame of compute: generateMortonCodes, sort, build, barnesHut,
    /// updateSpheres with the frame's dt (Renderer.swift:501-542).
    public func draw(dt: Float) throws {
        try check(astro_step(ctx, dt, 1))
    }

    /// Positions and velocities back for rendering.
    public func download(_ positions: inout [PositionMass], _ velocities: inout [VelocityRadius]) throws {
        let n = UInt32(positions.count)
        try positions.withUnsafeMutableBufferPointer { p in
            try velocities.withUnsafeMutableBufferPointer { v in
                try check(astro_download(ctx, p.baseAddress, v.baseAddress, n))
            }
        }
    }

    private func check(_ status: Int32) throws {
        if status != 0 {
            let msg = ctx.flatMap { String(cString: astro_last_error($0)) } ?? ""
            throw AstroError.status(status, msg)
        }
    }
}
