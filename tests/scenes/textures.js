{
   /* Image maps: a checker kd map repeated on the floor (Lanczos filter), a bump-mapped back
    * wall, a Phong cube with a ks map (cube uvs) and a diffuse OBJ mesh with the checker, under
    * a unit-plane light, in a Radiance HDR environment seen through the open sides.
    * make_textures.py writes checker.png, bumps.ppm and sky.hdr. */
   "scenefile" : {
      "renderer" : { "type" : "pathTracer", "noSuperSamples" : 16, "noDirectSamples" : 2,
                     "maxDepth" : 5, "rrStartDepth" : 3, },
      "camera" : { "type" : "pinhole", "eye" : [ 0, 1, 3.6 ], "look" : [ 0, -0.05, -1 ], "up" : [ 0, 1, 0 ],
                   "heightAngle" : 42, },
      "output" : { "width" : 40, "height" : 40, },
      "scene" : {
         "background" : { "emitter" : { "type" : "environment", "path" : "sky.hdr", }, },
         "material" : {
            "repeatU" : 3, "repeatV" : 2,
            "filter" : { "type" : "lanczosSinc", "support" : 3, "tau" : 2 },
            "bsdf" : { "type" : "diffuse", "kd" : "checker.png", },
            "plane" : { "vertices" : [ -1, 0, 1,   1, 0, 1,   1, 0, -1,   -1, 0, -1 ], },
         },
         "material" : {
            "bumpMap" : "bumps.ppm", "bumpIntensity" : 4,
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.6, 0.6, 0.55 ], },
            "plane" : { "vertices" : [ -1, 0, -1,   1, 0, -1,   1, 2, -1,   -1, 2, -1 ], },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : [ 0.5, 0.3, 0.3 ], },
            "plane" : { "vertices" : [ -1, 0, 1,   -1, 0, -1,   -1, 2, -1,   -1, 2, 1 ], },
         },
         "material" : {
            "bsdf" : { "type" : "phong", "kd" : 0.3, "ks" : "checker.png", "n" : 25, },
            "transform" : {
               "translate" : [ -0.4, 0.3, -0.2 ],
               "rotate" : [ 0, 0, 0,  0, 1, 0,  30 ],
               "scale" : [ 0.6, 0.6, 0.6 ],
               "cube" : { },
            },
         },
         "material" : {
            "bsdf" : { "type" : "diffuse", "kd" : "checker.png", },
            "transform" : {
               "translate" : [ 0.45, 0.3, 0.3 ],
               "scale" : [ 0.3, 0.3, 0.3 ],
               "mesh" : { "path" : "octahedron.obj", },
            },
         },
         "material" : {
            "emitter" : { "type" : "oriented", "power" : [ 9, 9, 8 ], },
            "transform" : {
               "translate" : [ 0, 1.99, 0 ],
               "rotate" : [ 0, 0, 0,  1, 0, 0,  180 ],
               "scale" : [ 0.6, 1, 0.6 ],
               "plane" : { },
            },
         },
      },
   },
}
