// swift-tools-version:5.9
// Swift host for libastro_cuda (written for a Swift toolchain on Linux;
// build with: swift build -Xlinker -L../astro_gb300/lib).
import PackageDescription

let package = Package(
    name: "AstroHost",
    targets: [
        .systemLibrary(name: "CAstroCUDA", path: "Sources/CAstroCUDA"),
        .target(name: "AstroHost", dependencies: ["CAstroCUDA"], path: "Sources/AstroHost"),
    ]
)
