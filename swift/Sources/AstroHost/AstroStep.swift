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

    /// Colours after the lighting pass (BarnesHut.metal:103-167), which the
    /// REFERENCE step runs between barnesHut and updateSpheres.
    public func colors(count: Int) throws -> [ColorType] {
        var out = [ColorType](repeating: ColorType(), count: count)
        try out.withUnsafeMutableBufferPointer { c in
            try check(astro_read_colors(ctx, c.baseAddress, UInt32(count)))
        }
        return out
    }

    /// The scene pass drawn headless into RGBA floats (row 0 at the top) with
    /// the Renderer's view and projection matrices (column-major).
    public func splat(view: [Float], projection: [Float], camera: [Float],
                      width: UInt32, height: UInt32) throws -> [Float] {
        var cam = astro_camera()
        withUnsafeMutableBytes(of: &cam.view) { $0.copyBytes(from: view.withUnsafeBytes { Array($0) }) }
        withUnsafeMutableBytes(of: &cam.projection) { $0.copyBytes(from: projection.withUnsafeBytes { Array($0) }) }
        withUnsafeMutableBytes(of: &cam.position) { $0.copyBytes(from: camera.withUnsafeBytes { Array($0) }) }
        var rgba = [Float](repeating: 0, count: Int(width) * Int(height) * 4)
        try rgba.withUnsafeMutableBufferPointer { out in
            try check(astro_splat(ctx, &cam, width, height, nil, out.baseAddress, nil))
        }
        return rgba
    }

    /// resetSimulation / makeSpheres without regeneration: save and reload the
    /// state between frames.
    public func save(path: String, step: UInt64, time: Double) throws {
        try check(astro_save_state(ctx, path, step, time))
    }

    public static func load(path: String) throws -> (AstroStep, UInt64, Double) {
        var c: OpaquePointer?
        var step: UInt64 = 0
        var time: Double = 0
        let status = astro_load_state(path, 0, &c, &step, &time)
        if status != 0 { throw AstroError.status(status, "astro_load_state") }
        return (AstroStep(context: c), step, time)
    }

    private init(context: OpaquePointer?) { ctx = context }

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
